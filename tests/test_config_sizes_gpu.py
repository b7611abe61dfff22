"""GPU parity at the workloads' own sizes: the CUDA FP64 path against the CPU
oracle (the reference algorithm restated, itself pinned bit for bit to the
reference's kernels by the golden fixtures), where the other parity tests use
small systems.

* 1024 bidisperse disks at phi 0.80, velocities at T = 1e-4: 10^4 NVE steps of
  dt = 1e-2, bit-identical state; total energy (drift) equal to 1e-12.
* 16384 disks at phi 0.86: 500 FIRE iterations bit-identical, with the default
  force group (8 lanes per particle at this size) and with one lane.
* 4096 rigid bumpy bodies (20 / 28 vertices): setup forces and vertex lists
  bit-identical, 100 NVE steps to 1e-9 (vertex rotations use cos / sin, whose
  CUDA and host-libm results may differ in the last bit).
* 2^20 polydisperse disks (radii U[0.4, 0.6], phi 0.84): setup forces, energies
  and neighbour counts bit-identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
KEYS = ("x", "y", "vx", "vy", "fx", "fy", "pe")
CUT_MULT = 1.7 / 1.4


@pytest.fixture(scope="module")
def dpg():
    import dpcuda_gb300
    dpcuda_gb300.load_library()
    return dpcuda_gb300


def same(s, o, tag):
    a, b = s.getState(), o.get_arrays()
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{tag} {k}")


def thermal(n, T, seed):
    from oracle.oracle import fill_normal
    vx = fill_normal(n, 0.0, np.sqrt(T), 1, seed)
    vy = fill_normal(n, 0.0, np.sqrt(T), 1 + n, seed)
    return vx - vx.mean(), vy - vy.mean()


def test_nve_1024_disks_ten_thousand_steps(dpg):
    from oracle.oracle import DiskOracle, disk_packing
    n = 1024
    st = disk_packing(n, 0.80, 1)
    vx, vy = thermal(n, 1e-4, 1)
    o = DiskOracle(n, st["box"])
    o.set_arrays(x=st["x"], y=st["y"], vx=vx, vy=vy, r=st["r"], m=st["m"])
    o.setup_neighbors(0, CUT_MULT, 0.2, 8.0, 0.5)
    s = dpg.Disk(n, st["box"])
    s.setState(st["x"], st["y"], vx, vy, st["r"], st["m"])
    s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
    same(s, o, "setup")
    e0 = o.total_ke() + o.total_pe()
    for _ in range(10):
        s.nveSteps(1e-2, 1000)
        o.nve_steps(1e-2, 1000)
    same(s, o, "10^4 NVE steps")
    e_gpu = s.totalKineticEnergy() + s.totalPotentialEnergy()
    e_orc = o.total_ke() + o.total_pe()
    np.testing.assert_allclose(e_gpu, e_orc, rtol=1e-12)
    # the drift itself: velocity Verlet at dt = 1e-2 keeps the energy
    assert abs(e_orc / e0 - 1) < 1e-3
    info = s.neighborInfo()
    assert (info["n_rebuilds"], info["n_cell_rebuilds"]) == o.num_rebuilds()
    s.close()


@pytest.mark.parametrize("lanes", [0, 1])
def test_fire_16384_disks_500_iterations(dpg, lanes):
    from oracle.oracle import DiskOracle, disk_packing
    n = 16384
    st = disk_packing(n, 0.86, 1)
    o = DiskOracle(n, st["box"])
    o.set_arrays(x=st["x"], y=st["y"], r=st["r"], m=st["m"])
    o.setup_neighbors(0, CUT_MULT, 0.2, 8.0, 0.5)
    s = dpg.Disk(n, st["box"])
    s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
    s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
    if lanes:
        s.setForceGroup(lanes)
    same(s, o, "setup")
    # no stop test fires before 500 iterations at these targets
    r = dpg.minimizeFire(s, 0.1, 1e-2, 0.0, 0.0, 500)
    o.minimize_fire(0.1, 1e-2, 0.0, 0.0, 500, 0.0)
    assert r["steps"] == 500
    same(s, o, "500 FIRE iterations")
    s.close()


def test_rigid_bumpy_4096_bodies(dpg):
    from oracle.oracle import BumpyOracle, bumpy_packing
    nb = 4096
    st = bumpy_packing(nb, 0.80, 3)
    vx, vy = thermal(nb, 1e-4, 3)
    w = np.zeros(nb)
    o = BumpyOracle(nb, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], True)
    o.set_bodies(st["x"], st["y"], st["th"], st["r"], st["nvb"], vx, vy, w)
    o.init_vertices()
    o.set_mass(1.0)
    code = o.setup_neighbors(0, 1.5, 0.2, 8.0, 0.5)
    px, py = o.vertices()
    b = dpg.RigidBumpy(nb, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], True)
    b.setBodies(st["x"], st["y"], st["th"], st["r"], st["nvb"], vx, vy, w)
    b.setVertexPositions(px, py)
    b.setMass(1.0)
    assert b.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)["method"] == code
    g, r = b.getBodies(), o.bodies()
    for k in ("x", "y", "th", "vx", "vy", "w", "fx", "fy", "tq", "pe"):
        np.testing.assert_array_equal(g[k], r[k], err_msg=f"setup {k}")
    assert b.getVertexNeighborSets() == o.vertex_neighbor_sets()
    b.nveSteps(5e-3, 100)
    o.nve_steps(5e-3, 100)
    g, r = b.getBodies(), o.bodies()
    for k in ("x", "y", "th", "vx", "vy", "w", "fx", "fy", "tq", "pe"):
        np.testing.assert_allclose(g[k], r[k], rtol=0, atol=1e-9, err_msg=f"100 NVE steps {k}")
    b.close()


def test_setup_forces_two_to_the_twenty_disks(dpg):
    from dpcuda_gb300.init import random_uniform
    from oracle.oracle import DiskOracle
    n = 1 << 20
    r = random_uniform(n, 0.4, 0.6, 7 * n, 5)
    L = (float(np.sum(r * r)) * np.pi / 0.84) ** 0.5
    x = random_uniform(n, 0.0, L, 0, 5)
    y = random_uniform(n, 0.0, L, n, 5)
    m = np.ones(n)
    o = DiskOracle(n, L)
    o.set_arrays(x=x, y=y, r=r, m=m)
    o.setup_neighbors(0, 1.5 / 1.2, 0.1732, 8.0, 0.5)
    s = dpg.Disk(n, L)
    s.setState(x, y, None, None, r, m)
    s.setupNeighbors("cell", 1.5 / 1.2, 0.1732, 8.0, 0.5)
    a, b = s.getState(), o.get_arrays()
    for k in ("x", "y", "fx", "fy", "pe"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    s.close()

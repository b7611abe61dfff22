"""GPU: the CUDA FP64 path against the oracle over a sweep the fixtures do not
cover -- sizes 16 to 700, packing fractions 0.5 to 0.95, the cell, Verlet and
all-pairs methods -- through setup, NVE, FIRE, Adam and DampedNVE.  The FP64
path follows the reference's operation order, so positions, velocities,
forces and energies must agree bit for bit (FIRE's power is a grid reduction
on the GPU and a sequential sum in the oracle; its sign decides the FIRE
branch, and it is never near zero in these runs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
KEYS = ("x", "y", "vx", "vy", "fx", "fy", "pe")


@pytest.fixture(scope="module")
def dpg():
    import dpcuda_gb300
    dpcuda_gb300.load_library()
    return dpcuda_gb300


def same(s, o, tag):
    a, b = s.getState(), o.get_arrays()
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=f"{tag} {k}")


@pytest.mark.parametrize("n,phi,seed", [(16, 0.5, 1), (100, 0.85, 2), (333, 0.95, 3), (700, 0.7, 4)])
@pytest.mark.parametrize("method,name", [(0, "cell"), (1, "verlet"), (2, "all")])
def test_fp64_path_matches_oracle_across_sizes_and_methods(dpg, n, phi, seed, method, name):
    from oracle.oracle import DiskOracle, disk_packing, fill_normal
    st = disk_packing(n, phi, seed)
    vx = fill_normal(n, 0.0, 1e-2, 1, seed)
    vy = fill_normal(n, 0.0, 1e-2, 1 + n, seed)
    o = DiskOracle(n, st["box"])
    o.set_arrays(x=st["x"], y=st["y"], vx=vx, vy=vy, r=st["r"], m=st["m"])
    code = o.setup_neighbors(method, 1.7 / 1.4, 0.2, 8.0, 0.5)
    s = dpg.Disk(n, st["box"])
    s.setState(st["x"], st["y"], vx, vy, st["r"], st["m"])
    assert s.setupNeighbors(name, 1.7 / 1.4, 0.2, 8.0, 0.5)["method"] == code
    same(s, o, "setup")
    s.nveSteps(1e-2, 40)
    o.nve_steps(1e-2, 40)
    same(s, o, "nve")
    fire = dpg.Fire(s, 0.1, 1e-2)
    o.fire_init(0.1, 1e-2)
    for _ in range(30):
        fire.step()
        o.fire_step()
    same(s, o, "fire")
    s.initAdamVariables()
    adam = dpg.Adam(s, 1e-3, 0.9, 0.999, 1e-8)
    o.init_adam()
    for t in range(15):
        adam.minimize(t)
        o.zero_force_and_pe()
        o.check_for_neighbor_update()
        o.calculate_forces()
        o.adam_step(t, 1e-3)
    same(s, o, "adam")
    s.dampedNveSteps(1e-2, 0.3, 20)
    o.damped_nve_steps(1e-2, 0.3, 20)
    same(s, o, "damped")
    s.close()


@pytest.mark.parametrize("nb,phi,seed", [(8, 0.6, 11), (40, 0.85, 12), (150, 0.75, 13)])
@pytest.mark.parametrize("rotation", [True, False])
def test_rigid_path_matches_oracle_across_sizes(dpg, nb, phi, seed, rotation):
    """Rigid bodies: setup forces bit for bit (same vertex positions); NVE,
    FIRE, DampedNVE and Adam trajectories to 1e-9 (vertex rotations use
    cos / sin, whose CUDA and host-libm results may differ in the last bit)."""
    from oracle.oracle import BumpyOracle, bumpy_packing, fill_normal
    st = bumpy_packing(nb, phi, seed)
    vx = fill_normal(nb, 0.0, 1e-2, 1, seed)
    vy = fill_normal(nb, 0.0, 1e-2, 1 + nb, seed)
    w = fill_normal(nb, 0.0, 1e-2, 1 + 2 * nb, seed)
    o = BumpyOracle(nb, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], rotation)
    o.set_bodies(st["x"], st["y"], st["th"], st["r"], st["nvb"], vx, vy, w)
    o.init_vertices()
    o.set_mass(1.0)
    code = o.setup_neighbors(0, 1.5, 0.2, 8.0, 0.3)
    px, py = o.vertices()
    b = dpg.RigidBumpy(nb, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], rotation)
    b.setBodies(st["x"], st["y"], st["th"], st["r"], st["nvb"], vx, vy, w)
    b.setVertexPositions(px, py)
    b.setMass(1.0)
    assert b.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.3)["method"] == code

    def check(tag, exact=False):
        g, r = b.getBodies(), o.bodies()
        for k in ("x", "y", "th", "vx", "vy", "w", "fx", "fy", "tq", "pe"):
            if exact:
                np.testing.assert_array_equal(g[k], r[k], err_msg=f"{tag} {k}")
            else:
                np.testing.assert_allclose(g[k], r[k], rtol=0, atol=1e-9, err_msg=f"{tag} {k}")

    check("setup", exact=True)
    b.nveSteps(5e-3, 30)
    o.nve_steps(5e-3, 30)
    check("nve")
    b.fireInit(0.1, 1e-2)
    o.fire_init(0.1, 1e-2)
    for _ in range(25):
        b.fireStep()
        o.fire_step()
    check("fire")
    b.dampedNveSteps(5e-3, 0.4, 20)
    o.damped_nve_steps(5e-3, 0.4, 20)
    check("damped")
    b.initAdamVariables()
    for t in range(20):
        b.adamMinimizeStep(t, 2e-3)
    o.adam_steps(20, 2e-3)
    check("adam")
    b.close()

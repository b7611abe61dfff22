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

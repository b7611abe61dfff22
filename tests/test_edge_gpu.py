"""GPU edge cases of the FP64 drop-in and the batched form: the analytic
two-disk contact, a lone particle (no neighbours), the all-pairs and Verlet
neighbour methods at small N against the oracle (bit for bit), and ragged
ensembles with systems of 1, 2 and 3 particles."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
CUT_MULT = 1.7 / 1.4


@pytest.fixture(scope="module")
def dpg():
    import dpcuda_gb300
    dpcuda_gb300.load_library()
    return dpcuda_gb300


def test_two_disk_contact_known_answer(dpg):
    """Radii 0.5 at distance 0.9 in a box of 10: overlap 1 - 0.9 = 0.1, force
    e_c * overlap / sigma = 0.1 along the line of centres, energy per disk
    e_c * overlap^2 / 4 = 0.0025 (include/particles/base/kernels.cuh:154-183)."""
    s = dpg.Disk(2, 10.0)
    s.setState(np.array([4.0, 4.9]), np.array([5.0, 5.0]), None, None, np.array([0.5, 0.5]),
               np.ones(2))
    s.setupNeighbors("all", 1.5, 0.2, 8.0, 0.5)
    s.zeroForceAndPotentialEnergy()
    s.calculateForces()
    g = s.getState()
    np.testing.assert_allclose(g["fx"], [-0.1, 0.1], rtol=1e-14)
    np.testing.assert_array_equal(g["fy"], [0.0, 0.0])
    np.testing.assert_allclose(g["pe"], [0.0025, 0.0025], rtol=1e-14)
    assert g["fx"][0] == -g["fx"][1]  # Newton's third law, exactly
    s.close()


def test_lone_particle_moves_ballistically(dpg):
    from oracle.oracle import DiskOracle
    s = dpg.Disk(1, 20.0)
    s.setState(np.array([3.0]), np.array([4.0]), np.array([0.25]), np.array([-0.5]),
               np.array([0.5]), np.ones(1))
    s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
    s.nveSteps(1e-2, 1000)
    o = DiskOracle(1, 20.0)
    o.set_arrays(x=np.array([3.0]), y=np.array([4.0]), vx=np.array([0.25]), vy=np.array([-0.5]),
                 r=np.array([0.5]), m=np.ones(1))
    o.setup_neighbors(0, CUT_MULT, 0.2, 8.0, 0.5)
    o.nve_steps(1e-2, 1000)
    a, b = s.getState(), o.get_arrays()
    for k in ("x", "y", "vx", "vy", "fx", "fy", "pe"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert np.all(a["fx"] == 0.0) and np.all(a["pe"] == 0.0)
    s.close()


@pytest.mark.parametrize("method,code", [("all", 2), ("verlet", 1)])
def test_all_pairs_and_verlet_methods_bitexact(dpg, method, code):
    from oracle.oracle import DiskOracle, disk_packing
    st = disk_packing(100, 0.84, 17)
    s = dpg.Disk(100, st["box"])
    s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
    info = s.setupNeighbors(method, CUT_MULT, 0.2, 8.0, 0.5)
    assert info["method"] == code
    o = DiskOracle(100, st["box"])
    o.set_arrays(x=st["x"], y=st["y"], r=st["r"], m=st["m"])
    assert o.setup_neighbors(code, CUT_MULT, 0.2, 8.0, 0.5) == code
    s.nveSteps(1e-2, 200)
    o.nve_steps(1e-2, 200)
    a, b = s.getState(), o.get_arrays()
    for k in ("x", "y", "vx", "vy", "fx", "fy", "pe"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    s.close()


def test_ragged_ensemble_with_tiny_systems(dpg):
    """Systems of 1, 2, 3 and 64 disks in one ensemble: FP64 forces equal the
    plain path's, a lone disk has none, and a FIRE run finishes every system."""
    from oracle.oracle import disk_packing
    # dilute tiny systems (boxes wider than twice the cutoff, so the minimum
    # image is unambiguous), a dense 64-disk one
    sts = [disk_packing(n, 0.1 if n < 4 else 0.7, 90 + n) for n in (1, 2, 3, 64)]
    e = dpg.Ensemble([len(s["r"]) for s in sts], [s["box"] for s in sts], 1.7, 0.3,
                     precision=dpg.FP64)
    e.setState(*[np.concatenate([s[c] for s in sts]) for c in ("x", "y", "r", "m")])
    e.calculateForces(dpg.FP64)
    got = e.getState()
    off = 0
    for st in sts:
        n = len(st["r"])
        s = dpg.Disk(n, st["box"])
        s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
        s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        s.zeroForceAndPotentialEnergy()
        s.calculateForces()
        want = s.getState()
        scale = max(1.0, np.abs(want["fx"]).max())
        for c in ("fx", "fy"):
            np.testing.assert_allclose(got[c][off:off + n], want[c], rtol=0, atol=1e-12 * scale)
        off += n
        s.close()
    assert got["fx"][0] == 0.0 and got["fy"][0] == 0.0
    res = e.minimizeFire(0.1, 1e-2, 0.0, 0.0, 200_000, fmax_target=1e-12)
    assert all(r["converged"] == 1 and r["max_force"] <= 1e-12 for r in res), res
    e.close()

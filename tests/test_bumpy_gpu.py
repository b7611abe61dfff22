"""GPU parity of the rigid-bumpy path (warp-per-body kernels) against the
golden fixtures made by the reference's own bumpy kernels and the CPU oracle.

With identical vertex positions, vertex forces and the per-body sums are
bit-identical (the body sums run in vertex order through warp shuffles).  The
vertex rotation uses cos/sin, whose CUDA and host-libm results can differ in
the last bit, so trajectories are compared with a tolerance: 1e-9 absolute on
positions and forces after 60 FIRE steps.
"""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = Path(__file__).resolve().parent / "golden"
BODY = ("x", "y", "th", "vx", "vy", "w", "fx", "fy", "tq", "pe")


@pytest.fixture(scope="module")
def dpg():
    import dpcuda_gb300
    dpcuda_gb300.load_library()
    return dpcuda_gb300


def make(dpg, d, explicit_vertices=True):
    nb = len(d["r"])
    b = dpg.RigidBumpy(nb, int(d["nvb"].sum()), float(d["box"]), float(d["e_c"]), 2.0,
                       float(d["rv"]), float(d["seg"]), True)
    b.setBodies(d["x0"], d["y0"], d["th0"], d["r"], d["nvb"])
    if explicit_vertices:
        b.setVertexPositions(d["px0"], d["py0"])
    b.setMass(1.0)
    return b


@pytest.mark.parametrize("name", ["bumpy_n64_verlet.npz", "bumpy_n256_cell.npz"])
def test_vertex_placement_and_inertia(dpg, name):
    d = dict(np.load(G / name))
    b = make(dpg, d, explicit_vertices=False)
    px, py = b.getVertexPositions()
    np.testing.assert_allclose(px, d["px0"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(py, d["py0"], rtol=0, atol=1e-13)
    b2 = make(dpg, d)
    np.testing.assert_array_equal(b2.getBodies()["I"], d["I"])


@pytest.mark.parametrize("name", ["bumpy_n64_verlet.npz", "bumpy_n256_cell.npz"])
def test_setup_forces_and_vertex_lists_bitexact(dpg, name):
    d = dict(np.load(G / name))
    b = make(dpg, d)
    info = b.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
    assert info["method"] == int(d["method"])
    bd = b.getBodies()
    for k in BODY:
        np.testing.assert_array_equal(bd[k], d[f"setup_{k}"], err_msg=k)
    gold = [frozenset(int(u) for u in row if u >= 0) for row in d["setup_vneighbors"]]
    assert b.getVertexNeighborSets() == gold


@pytest.mark.parametrize("name", ["bumpy_n64_verlet.npz", "bumpy_n256_cell.npz"])
def test_fire_steps_match_reference(dpg, name):
    d = dict(np.load(G / name))
    b = make(dpg, d)
    b.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
    b.fireInit(0.1, 1e-2)
    for _ in range(60):
        b.fireStep()
    bd = b.getBodies()
    for k in ("x", "y", "th", "fx", "fy", "tq"):
        np.testing.assert_allclose(bd[k], d[f"fire60_{k}"], rtol=0, atol=1e-9, err_msg=k)
    px, py = b.getVertexPositions()
    np.testing.assert_allclose(px, d["fire60_px"], rtol=0, atol=1e-9)


def test_fused_loop_matches_single_steps(dpg):
    d = dict(np.load(G / "bumpy_n256_cell.npz"))
    a = make(dpg, d)
    a.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
    for _ in range(40):  # NVE::step with the rigid overrides
        a.updateVelocities(2.5e-3)
        a.updatePositions(5e-3)
        a.checkForNeighborUpdate()
        a.zeroForceAndPotentialEnergy()
        a.calculateForces()
        a.updateVelocities(2.5e-3)
    b = make(dpg, d)
    b.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
    b.nveSteps(5e-3, 40)
    x, y = a.getBodies(), b.getBodies()
    for k in BODY:
        np.testing.assert_array_equal(x[k], y[k], err_msg=k)


def test_bumpy_fire_to_residual_force_and_torque(dpg):
    from oracle.oracle import bumpy_packing
    st = bumpy_packing(128, 0.82, 9)
    b = dpg.RigidBumpy(128, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], True)
    b.setBodies(st["x"], st["y"], st["th"], st["r"], st["nvb"])
    b.setMass(1.0)
    b.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
    r = b.minimizeFire(0.1, 1e-2, 0.0, 0.0, 400000, fmax_target=1e-12, tmax_target=1e-12)
    obs = b.observables()
    assert r["converged"] == 1 and obs["max_force"] <= 1e-12 and obs["max_torque"] <= 1e-12


def test_bumpy_nve_energy_drift(dpg):
    from oracle.oracle import bumpy_packing, fill_normal
    st = bumpy_packing(512, 0.80, 4)
    b = dpg.RigidBumpy(512, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], True)
    vx = fill_normal(512, 0.0, 1e-2, 1, 4)
    vy = fill_normal(512, 0.0, 1e-2, 513, 4)
    b.setBodies(st["x"], st["y"], st["th"], st["r"], st["nvb"], vx - vx.mean(), vy - vy.mean())
    b.setMass(1.0)
    b.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
    o0 = b.observables()
    e0 = o0["pe"] + o0["ke"]
    b.nveSteps(5e-3, 2000)
    o1 = b.observables()
    e1 = o1["pe"] + o1["ke"]
    assert abs(e1 - e0) / abs(e0) < 1e-3


# ---- the mixed form: FP32 vertex pairs, FP64 torques and body sums ----------
def make_mixed(dpg, d):
    nb = len(d["r"])
    b = dpg.RigidBumpy(nb, int(d["nvb"].sum()), float(d["box"]), float(d["e_c"]), 2.0,
                       float(d["rv"]), float(d["seg"]), True, precision=1)
    b.setBodies(d["x0"], d["y0"], d["th0"], d["r"], d["nvb"])
    b.setVertexPositions(d["px0"], d["py0"])
    b.setMass(1.0)
    return b


def test_mixed_body_forces_match_fp64(dpg):
    d = dict(np.load(G / "bumpy_n256_cell.npz"))
    a, m = make(dpg, d), make_mixed(dpg, d)
    a.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
    m.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
    ba, bm = a.getBodies(), m.getBodies()
    scale = max(np.abs(ba["fx"]).max(), np.abs(ba["fy"]).max())
    for k in ("fx", "fy"):
        np.testing.assert_allclose(bm[k], ba[k], rtol=0, atol=1e-5 * scale, err_msg=k)
    np.testing.assert_allclose(bm["tq"], ba["tq"], rtol=0, atol=1e-5 * np.abs(ba["tq"]).max())


def test_mixed_bumpy_fire_refines_to_fp64_residual(dpg):
    from oracle.oracle import bumpy_packing
    st = bumpy_packing(128, 0.82, 9)
    b = dpg.RigidBumpy(128, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], True,
                       precision=1)
    b.setBodies(st["x"], st["y"], st["th"], st["r"], st["nvb"])
    b.setMass(1.0)
    b.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
    r = b.minimizeFire(0.1, 1e-2, 0.0, 0.0, 400000, fmax_target=1e-12, tmax_target=1e-12)
    obs = b.observables()
    assert r["converged"] == 1 and obs["max_force"] <= 1e-12 and obs["max_torque"] <= 1e-12

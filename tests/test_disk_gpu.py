"""GPU parity: the sm_103a FP64 disk path (through the C ABI) against the golden
fixtures made by the reference's own kernels and against the CPU oracle.

Per-particle FP64 arithmetic is compiled without FMA contraction and follows
the reference's operation order, so forces, neighbour sets, cell lists and
whole NVE / FIRE / Adam trajectories must be BIT-IDENTICAL to the reference.
Only totals from grid reductions (summation order differs) carry a tolerance:
1e-12 relative.
"""
import os
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G = Path(__file__).resolve().parent / "golden"
CUT_MULT = 1.7 / 1.4
KEYS = ("x", "y", "vx", "vy", "fx", "fy", "pe")
RTOL_SUM = 1e-12


@pytest.fixture(scope="module")
def dpg():
    import dpcuda_gb300
    dpcuda_gb300.load_library()
    return dpcuda_gb300


def load(name):
    return dict(np.load(G / name))


def make(dpg, d, method="cell"):
    n = len(d["r"])
    s = dpg.Disk(n, float(d["box"]))
    s.setState(d["x0"], d["y0"], d.get("vx0"), d.get("vy0"), d["r"], d["m"])
    info = s.setupNeighbors(method, CUT_MULT, 0.2, 8.0, 0.5)
    assert info["method"] == int(d["method"])
    return s


def assert_state(s, d, prefix):
    a = s.getState()
    for k in KEYS:
        np.testing.assert_array_equal(a[k], d[f"{prefix}_{k}"], err_msg=f"{prefix}_{k}")


def golden_sets(arr):
    return [frozenset(int(j) for j in row if j >= 0) for row in arr]


def oracle_for(d):
    from oracle.oracle import DiskOracle
    n = len(d["r"])
    o = DiskOracle(n, float(d["box"]))
    o.set_arrays(x=d["x0"], y=d["y0"], vx=d.get("vx0"), vy=d.get("vy0"), r=d["r"], m=d["m"])
    o.setup_neighbors(0, CUT_MULT, 0.2, 8.0, 0.5)
    return o


# ---------------------------------------------------------------------------
def test_setup_forces_neighbors_cells_bitexact(dpg):
    d = load("disk_n1024_cell.npz")
    s = make(dpg, d)
    info = s.neighborInfo()
    assert info["n_cells_dim"] == int(d["n_cells_dim"]) and info["capacity"] == int(d["cap"])
    assert_state(s, d, "setup")
    assert s.getNeighborSets() == golden_sets(d["setup_neighbors"])
    ci, cs, si = s.getCells()
    np.testing.assert_array_equal(ci, d["setup_cell_index"])
    np.testing.assert_array_equal(cs, d["setup_cell_start"])
    np.testing.assert_array_equal(si, d["setup_static_index"])
    np.testing.assert_allclose(s.getStressTensor(), d["setup_stress"], rtol=RTOL_SUM, atol=1e-18)
    assert s.getContactCount() == float(d["setup_contacts"])


def test_nve_trajectory_bitexact(dpg):
    d = load("disk_n1024_cell.npz")
    s = make(dpg, d)
    s.nveSteps(1e-2, 500)
    assert_state(s, d, "nve500")
    info = s.neighborInfo()
    assert (info["n_rebuilds"], info["n_cell_rebuilds"]) == tuple(int(v) for v in d["nve500_rebuilds"])
    np.testing.assert_allclose(s.totalPotentialEnergy(), float(d["nve500_total_pe"]), rtol=RTOL_SUM)
    np.testing.assert_allclose(s.totalKineticEnergy(), float(d["nve500_total_ke"]), rtol=RTOL_SUM)


def test_single_ops_match_fused_nve(dpg):
    """The drop-in per-method calls give the same trajectory as the fused loop."""
    d = load("disk_n1024_cell.npz")
    s = make(dpg, d)
    for _ in range(120):  # NVE::step spelled out (src/integrator/nve.cu:15-25)
        s.updateVelocities(0.5e-2)
        s.updatePositions(1e-2)
        s.checkForNeighborUpdate()
        s.zeroForceAndPotentialEnergy()
        s.calculateForces()
        s.updateVelocities(0.5e-2)
    f = make(dpg, d)
    f.nveSteps(1e-2, 120)
    a, b = s.getState(), f.getState()
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k])


def test_damped_nve_and_gradient_descent_bitexact(dpg):
    """DampedNVE::step and GradDesc::step against the reference kernels'
    trajectories, with neighbour rebuilds on the way."""
    d = load("disk_n512_damped_gd.npz")
    s = make(dpg, d)
    s.dampedNveSteps(1e-2, 0.5, 300)
    assert_state(s, d, "damped300")
    info = s.neighborInfo()
    assert (info["n_rebuilds"], info["n_cell_rebuilds"]) == tuple(int(v) for v in d["damped300_rebuilds"])
    s.gradDescSteps(1e-2, 200)
    assert_state(s, d, "gd200")
    info = s.neighborInfo()
    assert (info["n_rebuilds"], info["n_cell_rebuilds"]) == tuple(int(v) for v in d["gd200_rebuilds"])
    # the per-method form of DampedNVE::step gives the same trajectory
    a, b = make(dpg, d), make(dpg, d)
    for _ in range(40):
        a.updateVelocities(0.5e-2)
        a.updatePositions(1e-2)
        a.checkForNeighborUpdate()
        a.zeroForceAndPotentialEnergy()
        a.calculateDampedForces(0.5)
        a.calculateForces()
        a.updateVelocities(0.5e-2)
    b.dampedNveSteps(1e-2, 0.5, 40)
    sa, sb = a.getState(), b.getState()
    for k in KEYS:
        np.testing.assert_array_equal(sa[k], sb[k])


def test_wall_forces_and_wall_nve_bitexact(dpg):
    """calculateWallForces and NVE::wall_step against the reference kernels'
    results (walls at 0 and L, pair distances still periodic, as the reference)."""
    d = load("disk_n256_walls.npz")
    s = make(dpg, d)
    s.zeroForceAndPotentialEnergy()
    s.calculateWallForces()
    assert_state(s, d, "wall")
    s.nveWallSteps(1e-2, 300)
    assert_state(s, d, "wallnve300")
    # the per-method form of NVE::wall_step gives the same trajectory
    a, b = make(dpg, d), make(dpg, d)
    for _ in range(30):
        a.updateVelocities(0.5e-2)
        a.updatePositions(1e-2)
        a.checkForNeighborUpdate()
        a.zeroForceAndPotentialEnergy()
        a.calculateWallForces()
        a.calculateForces()
        a.updateVelocities(0.5e-2)
    b.nveWallSteps(1e-2, 30)
    sa, sb = a.getState(), b.getState()
    for k in KEYS:
        np.testing.assert_array_equal(sa[k], sb[k])


def test_pair_and_hessian_dump_bitexact(dpg):
    """calculateForceDistancePairs in the reference's layout ([slot * cap + k],
    current order): every array bit-identical to the reference kernels' except
    the separation angle, which comes from CUDA's atan2 (2 ulp of glibc's)."""
    d = load("disk_n256_pairs.npz")
    s = make(dpg, d)
    s.nveSteps(1e-2, 50)
    assert s.neighborInfo()["capacity"] == int(d["cap"])
    got = s.calculateForceDistancePairs()
    for k, v in got.items():
        if k == "angle":
            np.testing.assert_allclose(v, d["pairs_angle"], rtol=0, atol=2e-15)
        else:
            np.testing.assert_array_equal(v, d[f"pairs_{k}"], err_msg=k)


def test_fire_steps_bitexact(dpg):
    d = load("disk_n1024_cell.npz")
    s = make(dpg, d)
    s.nveSteps(1e-2, 500)
    fire = dpg.Fire(s, 0.1, 1e-2)
    for _ in range(300):
        fire.step()
    assert_state(s, d, "fire300")
    st = fire.state()
    np.testing.assert_array_equal([st["alpha"], st["dt"], st["n_good"], st["n_bad"], st["stopped"]],
                                  d["fire300_state"])


def test_adam_bitexact(dpg):
    d = load("disk_n1024_cell.npz")
    s = make(dpg, d)
    s.nveSteps(1e-2, 500)
    fire = dpg.Fire(s, 0.1, 1e-2)
    for _ in range(300):
        fire.step()
    s.initAdamVariables()
    adam = dpg.Adam(s, 1e-3, 0.9, 0.999, 1e-8)
    for k in range(40):
        adam.minimize(k)
    assert_state(s, d, "adam40")


def test_small_system_verlet_fallback_bitexact(dpg):
    d = load("disk_n64_verlet.npz")
    s = make(dpg, d)
    assert_state(s, d, "setup")
    assert s.getNeighborSets() == golden_sets(d["setup_neighbors"])
    s.nveSteps(1e-2, 200)
    assert_state(s, d, "nve200")
    fire = dpg.Fire(s, 0.1, 1e-2)
    for _ in range(100):
        fire.step()
    assert_state(s, d, "fire100")


def test_fire_minimize_matches_reference(dpg):
    """minimizeFire to the reference's own criteria (PE stationary): same
    minimum.  The device loop's PE reductions round differently from the
    reference's sequential sums, so the exit step may differ slightly."""
    d = load("disk_n2048_fire_min.npz")
    s = make(dpg, d)
    r = dpg.minimizeFire(s, 0.1, 1e-2, 1e-16, 1e-16, 100000)
    assert r["stopped"] == int(d["stopped"])
    assert abs(r["steps"] - int(d["steps"])) <= max(50, int(d["steps"]) // 100)
    np.testing.assert_allclose(r["avg_pe"], float(d["avg_pe"]), rtol=1e-10)
    # the PE-change test stops FIRE while particles still move by ~1e-7 per
    # step, so stopping a few steps apart leaves positions ~1e-7 apart
    a = s.getState()
    np.testing.assert_allclose(a["x"], d["x"], rtol=0, atol=2e-6)
    # pressure: the stop points differ by a few steps; 1e-8 relative
    np.testing.assert_allclose(s.getPressure(), float(d["pressure"]), rtol=1e-8)


def test_fire_minimize_first_steps_bitexact_with_oracle(dpg):
    """Before any PE-ratio test can fire, the device loop and the oracle take
    identical steps (checked after max_steps iterations)."""
    d = load("disk_n2048_fire_min.npz")
    s = make(dpg, d)
    o = oracle_for(d)
    r = dpg.minimizeFire(s, 0.1, 1e-2, 1e-16, 1e-16, 700)
    steps, _ = o.minimize_fire(0.1, 1e-2, 1e-16, 1e-16, 700, 0.0)
    assert r["steps"] == steps == 700
    a, b = s.getState(), o.get_arrays()
    for k in ("x", "y", "fx", "fy", "pe"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_fire_to_residual_force(dpg):
    """FIRE run past PE stagnation to max|F| <= 1e-13 (the added stop)."""
    from oracle.oracle import disk_packing
    st = disk_packing(1024, 0.86, 11)
    s = dpg.Disk(1024, st["box"])
    s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
    s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
    r = dpg.minimizeFire(s, 0.1, 1e-2, 0.0, 0.0, 200000, fmax_target=1e-13)
    assert r["converged"] == 1 and r["stopped"] == 0
    assert r["max_force"] <= 1e-13
    mx, bal = s.forceStats()
    assert mx <= 1e-13 and bal < 1e-12


def test_loop_modes_agree(dpg, monkeypatch):
    """Conditional-graph, chunked-graph and plain-stream loops: same result."""
    d = load("disk_n1024_cell.npz")
    out = {}
    for mode in ("cond", "graph", "stream"):
        monkeypatch.setenv("DPG_LOOP_MODE", mode)
        s = make(dpg, d)
        s.nveSteps(1e-2, 77)
        r = dpg.minimizeFire(s, 0.1, 1e-2, 1e-16, 1e-16, 333)
        out[mode] = (s.getState(), r["steps"])
    for mode in ("graph", "stream"):
        assert out[mode][1] == out["cond"][1]
        for k in KEYS:
            np.testing.assert_array_equal(out[mode][0][k], out["cond"][0][k])


def test_scale_save_revert_match_oracle(dpg):
    d = load("disk_n1024_cell.npz")
    s = make(dpg, d)
    o = oracle_for(d)
    s.setLastState()
    o.set_last_state()
    s.scaleToPackingFractionFull(0.9)
    o.scale_to_packing_fraction(0.9)
    assert tuple(s.getBoxSize()) == o.box()
    dpg.minimizeFire(s, 0.1, 1e-2, 1e-16, 1e-16, 200)
    o.minimize_fire(0.1, 1e-2, 1e-16, 1e-16, 200, 0.0)
    a, b = s.getState(), o.get_arrays()
    for k in ("x", "y", "fx", "fy"):
        np.testing.assert_array_equal(a[k], b[k])
    s.revertToLastState()
    o.revert_to_last_state()
    s.scaleBox(0.98)
    o.scale_box(0.98)
    dpg.minimizeFire(s, 0.1, 1e-2, 1e-16, 1e-16, 200)
    o.minimize_fire(0.1, 1e-2, 1e-16, 1e-16, 200, 0.0)
    a, b = s.getState(), o.get_arrays()
    for k in ("x", "y", "fx", "fy"):
        np.testing.assert_array_equal(a[k], b[k])
    assert tuple(s.getBoxSize()) == o.box()


def test_capacity_growth_mid_loop(dpg):
    """Compression raises neighbour counts past the capacity during a device
    loop: the loop halts, the host grows the list (power of two) and resumes;
    the trajectory equals the oracle's (which resizes the same way)."""
    from oracle.oracle import disk_packing
    st = disk_packing(512, 0.2, 5)
    s = dpg.Disk(512, st["box"])
    s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
    s.setupNeighbors("verlet", 2.5, 0.2, 8.0, 0.5)
    from oracle.oracle import DiskOracle
    o = DiskOracle(512, st["box"])
    o.set_arrays(x=st["x"], y=st["y"], r=st["r"], m=st["m"])
    o.setup_neighbors(1, 2.5, 0.2, 8.0, 0.5)
    cap0 = s.neighborInfo()["capacity"]
    assert cap0 == o.neighbor_info()["cap"]
    for phi in (0.5, 0.8, 0.95):
        s.scaleToPackingFractionFull(phi)
        o.scale_to_packing_fraction(phi)
        dpg.minimizeFire(s, 0.1, 1e-2, 1e-16, 1e-16, 150)
        o.minimize_fire(0.1, 1e-2, 1e-16, 1e-16, 150, 0.0)
    assert s.neighborInfo()["capacity"] > cap0
    assert s.neighborInfo()["capacity"] == o.neighbor_info()["cap"]
    a, b = s.getState(), o.get_arrays()
    for k in ("x", "y", "fx", "fy"):
        np.testing.assert_array_equal(a[k], b[k])


def test_large_n_properties(dpg):
    """N = 2^20 (the large-N configuration): Newton's third law, neighbour
    symmetry, and forces of sampled particles against a direct sum."""
    from oracle.oracle import fill_uniform
    n = 1 << 20
    rng = np.random.default_rng(5)
    r = rng.uniform(0.4, 0.6, n)
    area = float(np.sum(r * r)) * np.pi
    L = (area / 0.84) ** 0.5
    x = fill_uniform(n, 0.0, L, 0, 1)
    y = fill_uniform(n, 0.0, L, n, 1)
    s = dpg.Disk(n, L)
    s.setState(x, y, None, None, r, np.ones(n))
    info = s.setupNeighbors("cell", 1.5 / 1.2, 0.2, 8.0, 0.5)
    assert info["method"] == 0
    a = s.getState()
    assert abs(a["fx"].sum()) < 1e-9 * n and abs(a["fy"].sum()) < 1e-9 * n
    lst, cnt = s.getNeighbors()
    idx = rng.choice(n, 64, replace=False)
    rc = info["cutoff"]
    for i in idx:
        dx = x - x[i]
        dx -= L * np.round(dx / L)
        dy = y - y[i]
        dy -= L * np.round(dy / L)
        d2 = dx * dx + dy * dy
        want = set(np.nonzero(d2 < rc * rc)[0].tolist()) - {int(i)}
        assert set(lst[i, :cnt[i]].tolist()) == want
        for j in want:  # symmetric list
            assert i in set(lst[j, :cnt[j]].tolist())
        rs = r + r[i]
        m = (d2 < rs * rs) & (np.arange(n) != i)
        dd = np.sqrt(d2[m])
        fm = (1.0 - dd / rs[m]) / (rs[m] * dd)
        fx = np.sum(fm * (-dx[m]))
        np.testing.assert_allclose(a["fx"][i], fx, rtol=1e-9, atol=1e-13)
    s.nveSteps(1e-2, 50)
    b = s.getState()
    assert np.all(np.isfinite(b["x"]))


def test_state_files_round_trip_in_reference_layout(dpg, tmp_path):
    """dpg_write_state writes the reference's StateLog layout ("%.17e", x<TAB>y,
    static order); dpg_read_state loads it back bit for bit."""
    d = load("disk_n1024_cell.npz")
    s = make(dpg, d)
    s.nveSteps(1e-2, 50)
    s.writeState(tmp_path / "restart", step=50)
    st = s.getState()
    lines = (tmp_path / "restart" / "positions.dat").read_text().splitlines()
    assert lines[3] == f"{st['x'][3]:.17e}\t{st['y'][3]:.17e}"
    assert (tmp_path / "restart" / "step.dat").read_text() == "50"
    assert dpg.Disk.stateCount(tmp_path / "restart") == len(d["r"])
    t = dpg.Disk(len(d["r"]), 1.0)
    t.readState(tmp_path / "restart")
    np.testing.assert_array_equal(t.getBoxSize(), s.getBoxSize())
    got = t.getState()
    for k in ("x", "y", "vx", "vy"):
        np.testing.assert_array_equal(got[k], st[k])
    # the loaded state continues like the original
    t.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
    s2 = dpg.Disk(len(d["r"]), float(d["box"]))
    s2.setState(st["x"], st["y"], st["vx"], st["vy"], d["r"], d["m"])
    s2.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
    t.nveSteps(1e-2, 20)
    s2.nveSteps(1e-2, 20)
    a, b = t.getState(), s2.getState()
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k])


# ---- the mixed form (DPG_MIXED): FP32 pair forces, FP64 sums and integration ----
def make_mixed(dpg, d, method="cell"):
    n = len(d["r"])
    s = dpg.Disk(n, float(d["box"]), precision=dpg.MIXED)
    s.setState(d["x0"], d["y0"], d.get("vx0"), d.get("vy0"), d["r"], d["m"])
    s.setupNeighbors(method, CUT_MULT, 0.2, 8.0, 0.5)
    return s


def test_mixed_forces_match_fp64(dpg):
    """FP32 pair forces from cell-centre offsets agree with the FP64 forces to
    1e-5 of the largest force (FP32 rounding of O(1) offsets and radii)."""
    d = load("disk_n1024_cell.npz")
    a, b = make(dpg, d), make_mixed(dpg, d)
    for s in (a, b):
        s.zeroForceAndPotentialEnergy()
        s.calculateForces()
    fa, fb = a.getState(), b.getState()
    scale = max(np.abs(fa["fx"]).max(), np.abs(fa["fy"]).max())
    for k in ("fx", "fy"):
        np.testing.assert_allclose(fb[k], fa[k], rtol=0, atol=1e-5 * scale)
    np.testing.assert_allclose(b.totalPotentialEnergy(), a.totalPotentialEnergy(), rtol=1e-5)


def test_mixed_nve_tracks_fp64_and_conserves_energy(dpg):
    d = load("disk_n1024_cell.npz")
    a, b = make(dpg, d), make_mixed(dpg, d)
    e0 = b.totalPotentialEnergy() + b.totalKineticEnergy()
    a.nveSteps(1e-2, 100)
    b.nveSteps(1e-2, 100)
    sa, sb = a.getState(), b.getState()
    np.testing.assert_allclose(sb["x"], sa["x"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(sb["y"], sa["y"], rtol=0, atol=1e-6)
    b.nveSteps(1e-2, 2000)
    e1 = b.totalPotentialEnergy() + b.totalKineticEnergy()
    assert abs(e1 - e0) / abs(e0) < 1e-3


def test_mixed_fire_refines_to_fp64_residual(dpg):
    """Mixed FIRE switches to FP64 pair arithmetic and reaches max|F| <= 1e-12
    from a random start; from a start inside a basin (max|F| <= 1e-7, below the
    switch) it ends at the FP64 path's energy.  (From a shallower start the
    FP32 phase may cross a low barrier into a neighbouring minimum.)"""
    from oracle.oracle import disk_packing
    st = disk_packing(2048, 0.86, 31)
    m0 = dpg.Disk(2048, st["box"], precision=dpg.MIXED)
    m0.setState(st["x"], st["y"], None, None, st["r"], st["m"])
    m0.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
    r0 = dpg.minimizeFire(m0, 0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=1e-12)
    assert r0["converged"] and r0["max_force"] <= 1e-12
    s = dpg.Disk(2048, st["box"])
    s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
    s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
    dpg.minimizeFire(s, 0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=1e-7)
    g = s.getState()
    r64 = dpg.minimizeFire(s, 0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=1e-12)
    pe64 = s.totalPotentialEnergy()
    m = dpg.Disk(2048, st["box"], precision=dpg.MIXED)
    m.setState(g["x"], g["y"], None, None, st["r"], st["m"])
    m.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
    r = dpg.minimizeFire(m, 0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=1e-12)
    assert r64["max_force"] <= 1e-12
    assert r["converged"] and r["max_force"] <= 1e-12
    np.testing.assert_allclose(m.totalPotentialEnergy(), pe64, rtol=1e-10)


def test_force_groups_give_identical_forces_and_autotune_restores_state():
    """1, 2, 4 and 8 lanes per particle: bit-identical forces and energies; the
    autotuner picks one of them and leaves the forces as they were."""
    import dpcuda_gb300 as dpg
    from oracle.oracle import disk_packing
    st = disk_packing(3000, 0.86, 31)
    s = dpg.Disk(3000, st["box"])
    s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
    s.setupNeighbors("cell", 1.7 / 1.4, 0.2, 8.0, 0.5)
    ref = None
    for g in (1, 2, 4, 8):
        s.setForceGroup(g)
        s.zeroForceAndPotentialEnergy()
        s.calculateForces()
        got = s.getState()
        if ref is None:
            ref = got
        for k in ("fx", "fy", "pe"):
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"{k} lanes={g}")
    lanes, us = s.autotuneForceGroup(20)
    assert lanes in (1, 2, 4, 8) and all(v > 0 for v in us.values())
    after = s.getState()
    for k in ("fx", "fy", "pe", "x", "y"):
        np.testing.assert_array_equal(after[k], ref[k], err_msg=k)
    s.nveSteps(1e-2, 20)  # the loops run with the chosen group
    s.close()

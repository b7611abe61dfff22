"""GPU: the batched form (ensembles of independent systems) against the plain
single-system path, which is itself bit-identical to the reference.

* Forces: one FP64 force pass of the ensemble equals the plain path's forces to
  1e-12 of the largest force (the summation order over a particle's contacts
  differs), energies / pressure / contacts to 1e-12 relative; the FP32 pair
  forces of the mixed form agree to 1e-5 of the largest force.
* FIRE: started from the same partly relaxed states (max|F| <= 1e-5, inside
  one basin), FP64 and mixed ensembles reach max|F| <= 1e-12 at the plain
  path's energy to 1e-10 relative.  (From a random start the FIRE paths of
  any two summation orders part ways and may end in different minima of the
  jammed landscape, so energies are compared inside a basin.)
* Jamming: every system ends in the pressure band with the contact count of a
  jammed state; packing fractions of the mixed and FP64 ensembles and of the
  single-system driver are compared.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
CUT = 1.7  # d_max + skin 0.3


@pytest.fixture(scope="module")
def dpg():
    import dpcuda_gb300
    dpcuda_gb300.load_library()
    return dpcuda_gb300


def packings(sizes, phi, seed0):
    from oracle.oracle import disk_packing
    return [disk_packing(n, phi, seed0 + k) for k, n in enumerate(sizes)]


def make(dpg, sts, precision, switch=1e-6, form=0, threads=0, cut=CUT, skin=0.3):
    e = dpg.Ensemble([len(s["r"]) for s in sts], [s["box"] for s in sts], cut, skin,
                     precision=precision, switch_fmax=switch)
    e.setForm(form, threads)
    e.setState(np.concatenate([s["x"] for s in sts]), np.concatenate([s["y"] for s in sts]),
               np.concatenate([s["r"] for s in sts]), np.concatenate([s["m"] for s in sts]))
    return e


def single(dpg, st):
    s = dpg.Disk(len(st["r"]), st["box"])
    s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
    s.setupNeighbors("cell", CUT / 1.4, 0.2, 8.0, 0.5)
    return s


def split(e, arr):
    starts = np.concatenate([[0], np.cumsum(e.n)])
    return [arr[starts[k]:starts[k + 1]] for k in range(e.S)]


def test_ensemble_forces_match_plain_path(dpg):
    sizes = [64, 200, 513, 1024, 4096]
    sts = packings(sizes, 0.86, 20)
    e = make(dpg, sts, dpg.FP64)
    res64 = e.calculateForces(dpg.FP64)
    g64 = e.getState()
    res32 = e.calculateForces(dpg.MIXED)
    g32 = e.getState()
    from dpcuda_gb300.ensemble import DWORD
    resdw = e.calculateForces(DWORD)
    gdw = e.getState()
    for k, st in enumerate(sts):
        s = single(dpg, st)
        s.zeroForceAndPotentialEnergy()
        s.calculateForces()
        want = s.getState()
        scale = max(np.abs(want["fx"]).max(), np.abs(want["fy"]).max())
        for c in ("fx", "fy"):
            np.testing.assert_allclose(split(e, g64[c])[k], want[c], rtol=0, atol=1e-12 * scale,
                                       err_msg=f"FP64 {c} n={sizes[k]}")
            np.testing.assert_allclose(split(e, g32[c])[k], want[c], rtol=0, atol=1e-5 * scale,
                                       err_msg=f"mixed {c} n={sizes[k]}")
            # double-word FP32 (~48 bits): the refinement's forces
            np.testing.assert_allclose(split(e, gdw[c])[k], want[c], rtol=0, atol=1e-12 * scale,
                                       err_msg=f"double-word {c} n={sizes[k]}")
        pe = s.totalPotentialEnergy() / sizes[k]
        np.testing.assert_allclose(res64[k]["avg_pe"], pe, rtol=1e-12)
        np.testing.assert_allclose(res32[k]["avg_pe"], pe, rtol=1e-5)
        np.testing.assert_allclose(resdw[k]["avg_pe"], pe, rtol=1e-11)
        np.testing.assert_allclose(res64[k]["pressure"], s.getPressure(), rtol=1e-12)
        assert res64[k]["contacts"] == s.getContactCount()
        s.close()
    e.close()


FORMS = [(1, 0), (2, 128), (2, 512)]  # grid; persistent with 128 / 512 threads


@pytest.mark.parametrize("form,threads", FORMS)
@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_ensemble_fire_matches_plain_path_inside_a_basin(dpg, precision, form, threads):
    sizes = [64, 200, 513, 1024, 96]
    sts = packings(sizes, 0.86, 40)
    relaxed, want = [], []
    for st in sts:
        s = single(dpg, st)
        dpg.minimizeFire(s, 0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=1e-5)
        g = s.getState()
        r0 = dict(st, x=g["x"], y=g["y"])
        relaxed.append(r0)
        s.close()
        s = single(dpg, r0)
        r = dpg.minimizeFire(s, 0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=1e-12)
        assert r["max_force"] <= 1e-12
        want.append(s.totalPotentialEnergy() / len(st["r"]))
        s.close()
    e = make(dpg, relaxed, getattr(dpg, precision), form=form, threads=threads)
    res = e.minimizeFire(0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=1e-12)
    for r, w in zip(res, want):
        assert r["converged"] == 1 and r["max_force"] <= 1e-12
        np.testing.assert_allclose(r["avg_pe"], w, rtol=1e-10)
    e.close()


@pytest.mark.parametrize("form", [1, 2])
def test_ensemble_jamming_reaches_the_band(dpg, form):
    sizes = [64, 96, 128]
    sts = packings(sizes, 0.80, 60)
    band = (1e-4 * 0.99, 1e-4 * 1.01)
    fire = (0.1, 1e-2, 0.0, 0.0, 1_000_000, 1e-12)
    phi = {}
    for name, precision in (("mixed", 1), ("fp64", 0)):
        e = make(dpg, sts, precision, form=form)
        res = e.jam(*band, compression_rate=0.99, length_tolerance=1e-10, decompress_factor=1.01,
                    max_compression_steps=500, fire=fire)
        for n, r in zip(sizes, res):
            # status 0: ended inside the band with more than 2 contacts per disk
            assert r["status"] == 0 and band[0] <= r["pressure"] <= band[1]
            assert r["contacts"] > 2 * n
        phi[name] = np.array([r["packing_fraction"] for r in res])
        e.close()
    single_phi = []
    for st in sts:
        s = single(dpg, st)
        g = dpg.jamPressure(s, *band, compression_rate=0.99, length_tolerance=1e-10,
                            decompress_factor=1.01, max_compression_steps=500,
                            fire=fire, neighbors=("cell", CUT / 1.4, 0.2, 8.0, 0.5))
        assert band[0] <= g["pressure"] <= band[1]
        single_phi.append(g["packing_fraction"])
        s.close()
    single_phi = np.array(single_phi)
    print("phi_J mixed", phi["mixed"], "fp64", phi["fp64"], "single", single_phi)
    # jammed packing fractions of these small systems lie near 0.84
    for v in (phi["mixed"], phi["fp64"], single_phi):
        assert np.all((v > 0.80) & (v < 0.88))


def test_persistent_form_grows_overflowing_lists(dpg):
    """A cutoff of 5 puts ~50 disks in each list, above the initial capacity of
    32: the persistent launch stops at the list build, the host grows the
    lists and the systems resume; the minima equal the grid form's."""
    sizes = [300, 700, 64]
    sts = packings(sizes, 0.86, 80)
    out = {}
    for form in (1, 2):
        e = make(dpg, sts, dpg.FP64, form=form, cut=5.0, skin=3.6)
        res = e.minimizeFire(0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=1e-12)
        assert all(r["converged"] == 1 and r["max_force"] <= 1e-12 for r in res), res
        out[form] = [r["avg_pe"] for r in res]
        e.close()
    # from random starts the two forms' roundings may lead to different minima;
    # both must be minima, and most systems land in the same one
    same = sum(abs(a - b) <= 1e-10 * max(abs(a), 1e-300) for a, b in zip(out[1], out[2]))
    assert same >= 1


def test_autotune_restores_positions_and_picks_a_form(dpg):
    sizes = [64, 200, 513, 1024]
    sts = packings(sizes, 0.86, 90)
    e = make(dpg, sts, dpg.MIXED)
    x0 = e.getState()["x"].copy()
    t = e.autotune(iters=100)
    # 3 skins x (grid, persistent 128 / 256 / 512, resident)
    assert t["form"] in ("grid", "persist", "resident") and len(t["candidates"]) == 15
    assert all(c["rate"] > 0 for c in t["candidates"])
    assert t["skin"] in {c["skin"] for c in t["candidates"]}
    np.testing.assert_array_equal(e.getState()["x"], x0)
    res = e.minimizeFire(0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=1e-12)
    assert all(r["converged"] == 1 and r["max_force"] <= 1e-12 for r in res)
    e.close()


def test_launch_count_follows_the_forms(dpg):
    """dpg_ensemble_launch_count: the resident form issues one launch per size
    class and time slice, the grid form one graph launch per loop segment
    (2^24 iterations), so a short solve of three size classes costs three
    resident launches and one graph launch."""
    from dpcuda_gb300.ensemble import FORM_GRID, FORM_RESIDENT
    sts = packings([100, 600, 3000], 0.86, 40)
    for form, expect in ((FORM_RESIDENT, 3), (FORM_GRID, 1)):
        e = make(dpg, sts, dpg.MIXED, form=form)
        e.minimizeFire(0.1, 1e-2, 0.0, 0.0, 50, fmax_target=1e-13)
        n0 = e.launchCount()
        e.setState(np.concatenate([s["x"] for s in sts]), np.concatenate([s["y"] for s in sts]),
                   np.concatenate([s["r"] for s in sts]), np.concatenate([s["m"] for s in sts]))
        e.minimizeFire(0.1, 1e-2, 0.0, 0.0, 200, fmax_target=1e-13)
        issued = e.launchCount() - n0
        e.close()
        assert issued >= expect
        assert issued < expect + 12   # plus the setup kernels of one solve


def test_state_round_trips_in_input_order(dpg):
    """setState orders each system's slots by cell (a spatial sort); getState
    returns positions in the caller's order, bit for bit (unwrapped
    coordinates included), and a force pass's forces follow the same order."""
    sts = packings([70, 1000, 4000], 0.86, 60)
    rng = np.random.default_rng(5)
    shifted = [dict(st, x=st["x"] + st["box"] * rng.integers(-2, 3, len(st["x"])))
               for st in sts]
    e = make(dpg, shifted, dpg.FP64)
    out = e.getState()
    e.close()
    assert np.array_equal(out["x"], np.concatenate([s["x"] for s in shifted]))
    assert np.array_equal(out["y"], np.concatenate([s["y"] for s in shifted]))
    e = make(dpg, sts, dpg.FP64)
    e.calculateForces(dpg.FP64)
    got = e.getState()
    for k, st in enumerate(sts):
        s = single(dpg, st)
        s.zeroForceAndPotentialEnergy()
        s.calculateForces()
        want = s.getState()
        s.close()
        scale = np.abs(want["fx"]).max()
        for c in ("fx", "fy"):
            np.testing.assert_allclose(split(e, got[c])[k], want[c], rtol=0, atol=1e-12 * scale)
    e.close()

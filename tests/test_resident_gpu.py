"""GPU: the resident form of the batched loop (one block, or a cluster of
blocks, per system holding it on chip) against the CPU oracle.

The resident form runs its own arithmetic (positions as FP64 cell centres plus
double-word offsets, double-word pair forces, FP64 passes only to certify), so
its trajectories differ from the other forms'; what it must deliver is a state
the reference arithmetic confirms:
* FIRE: every system of an uneven ensemble covering every size class (lanes per
  particle, one block, clusters of 2, 4 and 8 blocks) converges, and the
  oracle's FP64 forces at the final positions have max|F| <= 1e-13 (the FP64
  certification uses Newton reciprocals, the oracle IEEE division: 1 % slack),
  with the reported energy equal to the oracle's to 1e-12 relative;
* the same holds in FP64 precision;
* results do not depend on where the time-sliced launches end: two runs give
  bit-identical positions;
* jamming ends every system inside the pressure band, and the FP64 drop-in,
  minimising again at the final box, confirms the band;
* neighbour lists that overflow the initial capacity are grown and the run
  finishes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
CUT = 1.7  # d_max + skin 0.3
FMAX = 1e-13
SIZES = [64, 100, 200, 400, 900, 1500, 3000]


@pytest.fixture(scope="module")
def dpg():
    import dpcuda_gb300
    dpcuda_gb300.load_library()
    return dpcuda_gb300


def packings(sizes, phi, seed0):
    from oracle.oracle import disk_packing
    return [disk_packing(n, phi, seed0 + k) for k, n in enumerate(sizes)]


def make(dpg, sts, precision, cut=CUT, skin=0.3):
    from dpcuda_gb300.ensemble import FORM_RESIDENT
    e = dpg.Ensemble([len(s["r"]) for s in sts], [s["box"] for s in sts], cut, skin,
                     precision=precision, switch_fmax=1e-6)
    e.setForm(FORM_RESIDENT)
    e.setState(*[np.concatenate([s[c] for s in sts]) for c in ("x", "y", "r", "m")])
    return e


def oracle_forces(st, x, y, box=None):
    from oracle.oracle import DiskOracle
    o = DiskOracle(len(st["r"]), st["box"] if box is None else box)
    o.set_arrays(x=x, y=y, r=st["r"], m=st["m"])
    o.setup_neighbors(0, CUT / 1.4, 0.2, 8.0, 0.5)
    o.zero_force_and_pe()
    o.calculate_forces()
    a = o.get_arrays()
    pe = o.total_pe() / len(st["r"])
    o.close()
    return float(np.sqrt(a["fx"] ** 2 + a["fy"] ** 2).max()), pe


def check_minima(e, sts, res):
    fin = e.getState()
    off = 0
    for st, r in zip(sts, res):
        n = len(st["r"])
        assert r["converged"] == 1 and r["max_force"] <= FMAX, r
        f64, pe = oracle_forces(st, fin["x"][off:off + n], fin["y"][off:off + n])
        assert f64 <= 1.01 * FMAX, (n, f64)
        np.testing.assert_allclose(r["avg_pe"], pe, rtol=1e-12, err_msg=f"n={n}")
        off += n


@pytest.mark.parametrize("precision", ["MIXED", "FP64"])
def test_resident_fire_minima_pass_the_oracle(dpg, precision):
    sizes = SIZES if precision == "MIXED" else SIZES[:5]
    sts = packings(sizes, 0.86, 300)
    e = make(dpg, sts, getattr(dpg, precision))
    res = e.minimizeFire(0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=FMAX)
    check_minima(e, sts, res)
    if precision == "MIXED":
        # double words did the refinement, FP64 only certified
        assert all(r["dw_steps"] > 0 for r in res)
        assert all(r["fp64_steps"] <= 20 for r in res), [r["fp64_steps"] for r in res]
    e.close()


def test_resident_runs_are_reproducible(dpg):
    sts = packings([150, 700, 2500], 0.86, 320)
    out = []
    for _ in range(2):
        e = make(dpg, sts, dpg.MIXED)
        res = e.minimizeFire(0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=FMAX)
        out.append((e.getState(), [r["fire_steps"] for r in res]))
        e.close()
    assert out[0][1] == out[1][1]
    for c in ("x", "y", "fx", "fy"):
        np.testing.assert_array_equal(out[0][0][c], out[1][0][c], err_msg=c)


def test_resident_jamming_ends_in_the_band(dpg):
    sizes = [64, 200, 1100]
    sts = packings(sizes, 0.80, 340)
    P = 1e-4
    band = (0.99 * P, 1.01 * P)
    fire = (0.1, 1e-2, 1e-16, 0.0, 100000, FMAX)
    e = make(dpg, sts, dpg.MIXED)
    res = e.jam(*band, compression_rate=0.99, length_tolerance=1e-10, decompress_factor=1.01,
                max_compression_steps=2000, fire=fire)
    fin = e.getState()
    off = 0
    for st, r in zip(sts, res):
        n = len(st["r"])
        assert r["status"] == 0 and band[0] <= r["pressure"] <= band[1], r
        assert r["contacts"] > 2 * n
        assert 0.80 < r["packing_fraction"] < 0.88
        # the FP64 drop-in at the final box confirms the band
        d = dpg.Disk(n, r["box_length"])
        d.setState(fin["x"][off:off + n], fin["y"][off:off + n], None, None, st["r"], st["m"])
        d.setupNeighbors("cell", CUT / 1.4, 0.2, 8.0, 0.5)
        dpg.minimizeFire(d, *fire)
        assert band[0] <= d.getPressure() <= band[1]
        assert d.getContactCount() > 2 * n
        d.close()
        off += n
    e.close()


def test_resident_grows_overflowing_lists(dpg):
    """A cutoff of 5 puts ~50 disks in each list, above the initial capacity of
    32: the launch stops at the list build, the host grows the lists and every
    system resumes."""
    sts = packings([300, 1200, 64], 0.86, 360)
    e = make(dpg, sts, dpg.MIXED, cut=5.0, skin=3.6)
    res = e.minimizeFire(0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=FMAX)
    check_minima(e, sts, res)
    e.close()

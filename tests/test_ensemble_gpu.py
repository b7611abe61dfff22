"""GPU: the batched form (ensembles of independent systems) against per-system
runs.  FP64 ensembles use the reference pair arithmetic; mixed ensembles use
FP32 pair forces then an FP64 refinement.  Minimised energies must agree with
per-system FP64 minimisations to 1e-9 relative, residual forces must reach the
target, and jammed packing fractions must agree within 1e-6."""
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


def make(dpg, sts, precision, switch=1e-7):
    e = dpg.Ensemble([len(s["r"]) for s in sts], [s["box"] for s in sts], CUT, 0.3,
                     precision=precision, switch_fmax=switch)
    e.setState(np.concatenate([s["x"] for s in sts]), np.concatenate([s["y"] for s in sts]),
               np.concatenate([s["r"] for s in sts]), np.concatenate([s["m"] for s in sts]))
    return e


def single(dpg, st, fmax):
    s = dpg.Disk(len(st["r"]), st["box"])
    s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
    s.setupNeighbors("cell", CUT / 1.4, 0.2, 8.0, 0.5)
    r = dpg.minimizeFire(s, 0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=fmax)
    return r, s


@pytest.mark.parametrize("precision", [0, 1])
def test_ensemble_fire_matches_single_systems(dpg, precision):
    sizes = [64, 200, 513, 1024, 96]
    sts = packings(sizes, 0.86, 40)
    e = make(dpg, sts, precision)
    res = e.minimizeFire(0.1, 1e-2, 0.0, 0.0, 1_000_000, fmax_target=1e-12)
    for st, r in zip(sts, res):
        assert r["converged"] == 1 and r["max_force"] <= 1e-12
        ref, _ = single(dpg, st, 1e-12)
        # same minimum of the same landscape (FIRE paths may differ slightly)
        np.testing.assert_allclose(r["avg_pe"], ref["avg_pe"], rtol=1e-9)


def test_ensemble_jamming_matches_single_system_drivers(dpg):
    sizes = [64, 96, 128]
    sts = packings(sizes, 0.80, 60)
    band = (1e-4 * 0.99, 1e-4 * 1.01)
    fire = (0.1, 1e-2, 0.0, 0.0, 1_000_000, 1e-12)
    for precision in (1, 0):
        e = make(dpg, sts, precision)
        res = e.jam(*band, compression_rate=0.99, length_tolerance=1e-10, decompress_factor=1.01,
                    max_compression_steps=500, fire=fire)
        for st, r in zip(sts, res):
            s = dpg.Disk(len(st["r"]), st["box"])
            s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
            s.setupNeighbors("cell", CUT / 1.4, 0.2, 8.0, 0.5)
            g = dpg.jamPressure(s, *band, compression_rate=0.99, length_tolerance=1e-10,
                                decompress_factor=1.01, max_compression_steps=500,
                                fire=fire, neighbors=("cell", CUT / 1.4, 0.2, 8.0, 0.5))
            assert r["status"] == 0 and band[0] <= r["pressure"] <= band[1]
            assert abs(r["packing_fraction"] - g["packing_fraction"]) <= 1e-6

"""GPU jamming drivers (run-script control flow over the C ABI) against the
oracle's restatement of the same scripts: jammed packing fraction within 1e-6
(the tolerance the drop-in must meet)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dpg():
    import dpcuda_gb300
    dpcuda_gb300.load_library()
    return dpcuda_gb300


def systems(dpg, n, seed):
    from oracle.oracle import DiskOracle, disk_packing
    st = disk_packing(n, 0.80, seed)
    s = dpg.Disk(n, st["box"])
    s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
    s.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
    o = DiskOracle(n, st["box"])
    o.set_arrays(x=st["x"], y=st["y"], r=st["r"], m=st["m"])
    o.setup_neighbors(0, 1.5, 0.2, 8.0, 0.5)
    return s, o


@pytest.mark.parametrize("n,seed", [(64, 2), (96, 4)])
def test_pressure_band_jamming_matches_oracle(dpg, n, seed):
    from oracle.oracle import jam_pressure
    s, o = systems(dpg, n, seed)
    band = (1e-4 * 0.99, 1e-4 * 1.01)
    g = dpg.jamPressure(s, *band, compression_rate=0.99, length_tolerance=1e-10,
                        decompress_factor=1.01, max_compression_steps=500,
                        neighbors=("cell", 1.5, 0.2, 8.0, 0.5))
    c = jam_pressure(o, *band, compression_rate=0.99, length_tol=1e-10, decompress=1.01,
                     max_steps=500, neighbors=(0, 1.5, 0.2, 8.0, 0.5))
    assert g["status"] == c["status"] == 0
    assert band[0] <= g["pressure"] <= band[1]
    assert abs(g["packing_fraction"] - c["packing_fraction"]) <= 1e-6
    assert g["contacts"] > 2 * n


def test_energy_bisection_jamming_matches_oracle(dpg):
    from oracle.oracle import jam_phi
    s, o = systems(dpg, 64, 2)
    g = dpg.jamPhi(s, 1e-16, 1e-16, 1e-7, 1e-2, 1e-7, 500)
    c = jam_phi(o, 1e-16, 1e-16, 1e-7, 1e-2, 1e-7, 500)
    assert g["status"] == c["status"] == 0
    assert abs(g["packing_fraction"] - c["packing_fraction"]) <= 1e-6

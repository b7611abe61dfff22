"""CPU: the rigid-bumpy oracle (oracle/dpg_oracle_bumpy.c) reproduces the golden
fixtures made by the reference's own bumpy kernels, bit for bit."""
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import BumpyOracle

G = Path(__file__).resolve().parent / "golden"
BODY = ("x", "y", "th", "vx", "vy", "w", "fx", "fy", "tq", "pe")


def make(d):
    nb = len(d["r"])
    b = BumpyOracle(nb, int(d["nvb"].sum()), float(d["box"]), float(d["e_c"]), 2.0,
                    float(d["rv"]), float(d["seg"]), True)
    b.set_bodies(d["x0"], d["y0"], d["th0"], d["r"], d["nvb"])
    b.init_vertices()
    b.set_mass(1.0)
    return b


def check(b, d, prefix):
    bd = b.bodies()
    for k in BODY:
        np.testing.assert_array_equal(bd[k], d[f"{prefix}_{k}"], err_msg=f"{prefix}_{k}")
    px, py = b.vertices()
    np.testing.assert_array_equal(px, d[f"{prefix}_px"])
    np.testing.assert_array_equal(py, d[f"{prefix}_py"])


@pytest.mark.parametrize("name", ["bumpy_n64_verlet.npz", "bumpy_n256_cell.npz"])
def test_bumpy_oracle_matches_reference_kernels(name):
    d = dict(np.load(G / name))
    b = make(d)
    px, py = b.vertices()
    np.testing.assert_array_equal(px, d["px0"])
    np.testing.assert_array_equal(b.bodies()["I"], d["I"])
    assert b.setup_neighbors(0, 1.5, 0.2, 8.0, 0.5) == int(d["method"])
    check(b, d, "setup")
    gold = [frozenset(int(u) for u in row if u >= 0) for row in d["setup_vneighbors"]]
    assert b.vertex_neighbor_sets() == gold
    b.fire_init(0.1, 1e-2)
    for _ in range(60):
        b.fire_step()
    check(b, d, "fire60")
    info = b.neighbor_info()
    assert [info["n_rebuilds"], info["n_cell_rebuilds"]] == list(d["fire60_info"])

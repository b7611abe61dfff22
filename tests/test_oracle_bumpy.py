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


def extras_system(d, cdm=0.5):
    nb = len(d["r"])
    b = BumpyOracle(nb, int(d["nvb"].sum()), float(d["box"]), float(d["e_c"]), 2.0,
                    float(d["rv"]), float(d["seg"]), True)
    b.set_bodies(d["x0"], d["y0"], d["th0"], d["r"], d["nvb"], d["vx0"], d["vy0"], d["w0"])
    b.init_vertices()
    b.set_mass(1.0)
    assert b.setup_neighbors(0, 1.5, 0.2, 8.0, cdm) == int(d["method"])
    return b


def check_bodies(b, d, prefix, vertices=True):
    bd = b.bodies()
    for k in BODY:
        np.testing.assert_array_equal(bd[k], d[f"{prefix}_{k}"], err_msg=f"{prefix}_{k}")
    if vertices:
        px, py = b.vertices()
        np.testing.assert_array_equal(px, d[f"{prefix}_px"])
        np.testing.assert_array_equal(py, d[f"{prefix}_py"])


def counts(b):
    i = b.neighbor_info()
    return [i["n_rebuilds"], i["n_cell_rebuilds"]]


def test_bumpy_oracle_extras_match_reference_kernels():
    """Pair and Hessian dump, stress, contacts, walls, DampedNVE, Adam across re-sorts and
    setLastState / revertToLastState across re-sorts: bit for bit."""
    d = dict(np.load(G / "bumpy_n128_extras.npz"))
    b = extras_system(d)
    check_bodies(b, d, "setup")
    tot, per = b.stress()
    np.testing.assert_array_equal(tot, d["stress_tot"])
    np.testing.assert_array_equal(per, d["stress_body"])
    tot, cc, vcc = b.count_contacts()
    assert tot == float(d["contacts_tot"])
    np.testing.assert_array_equal(cc, d["contacts_body"])
    np.testing.assert_array_equal(vcc, d["vcontacts_body"])
    for k, v in b.pair_dump().items():
        np.testing.assert_array_equal(v, d[f"pairs_{k}"], err_msg=f"pairs_{k}")
    b.zero()
    b.wall_only()
    check_bodies(b, d, "wallonly", vertices=False)
    b.zero()
    b.wall_and_pair_forces()
    check_bodies(b, d, "wallpair", vertices=False)

    b = extras_system(d)
    b.damped_nve_steps(5e-3, 0.5, 200)
    check_bodies(b, d, "damped")
    assert counts(b) == list(d["damped_info"])

    b = extras_system(d)
    b.nve_wall_steps(5e-3, 200)
    check_bodies(b, d, "walls")
    assert counts(b) == list(d["walls_info"])

    b = extras_system(d, 0.05)
    b.adam_steps(150, 1e-2)
    check_bodies(b, d, "adam")
    assert counts(b) == list(d["adam_info"])

    b = extras_system(d, 0.05)
    b.save_state()
    b.fire_init(0.1, 1e-2)
    for _ in range(100):
        b.fire_step()
    assert counts(b) == list(d["revert_pre_info"])
    b.restore_state()
    check_bodies(b, d, "revert")
    b.zero()
    b.calculate_forces()
    check_bodies(b, d, "revertf", vertices=False)
    assert counts(b) == list(d["revert_info"])


def test_bumpy_two_body_stress_and_contacts_known_answer():
    """Two one-vertex bodies at rest whose vertices overlap: one contact each,
    one vertex contact each, and the virial of a single harmonic pair:
    sigma_xx = d * F / A with F = e_c (1 - d / 2 r_v) / (2 r_v) on each side
    (half of each body's term, summed over both bodies)."""
    rv, box, e_c = 0.5, 10.0, 1.0
    b = BumpyOracle(2, 2, box, e_c, 2.0, rv, 0.9, True)
    x = np.array([4.0, 4.9])
    b.set_bodies(x, np.array([5.0, 5.0]), np.zeros(2), np.array([rv, rv]), np.array([1, 1]))
    b.set_vertices(x, np.array([5.0, 5.0]))
    b.set_mass(1.0)
    b.setup_neighbors(2, 1.5, 0.2, 8.0, 0.5)
    tot, cc, vcc = b.count_contacts()
    assert tot == 2.0 and list(cc) == [1, 1] and list(vcc) == [1, 1]
    t, _ = b.stress()
    f = e_c * (1 - 0.9 / (2 * rv)) / (2 * rv)
    np.testing.assert_allclose(t[0], 0.9 * f / box**2, rtol=1e-14)
    assert t[1] == 0.0 and t[2] == 0.0 and t[3] == 0.0

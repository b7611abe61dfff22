"""CPU: the oracle (oracle/dpg_oracle.c) reproduces the golden fixtures that the
reference's own kernels produced (tests/golden/make_golden.py), bit for bit.

This pins the oracle; the GPU tests then compare the CUDA path against it.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import DiskOracle, fill_normal, fill_uniform, reference_available

G = Path(__file__).resolve().parent / "golden"
CUT_MULT = 1.7 / 1.4
KEYS = ("x", "y", "vx", "vy", "fx", "fy", "pe")


def load(name):
    return dict(np.load(G / name))


def make(d, kind="oracle"):
    n = len(d["r"])
    o = DiskOracle(n, float(d["box"]), kind=kind)
    vx = d.get("vx0")
    vy = d.get("vy0")
    o.set_arrays(x=d["x0"], y=d["y0"], vx=vx, vy=vy, r=d["r"], m=d["m"])
    meth = o.setup_neighbors(0, CUT_MULT, 0.2, 8.0, 0.5)
    assert meth == int(d["method"])
    return o


def assert_state(o, d, prefix):
    a = o.get_arrays()
    for k in KEYS:
        np.testing.assert_array_equal(a[k], d[f"{prefix}_{k}"], err_msg=f"{prefix}_{k}")


def static_neighbors(o):
    sets = o.static_neighbor_sets()
    return [sorted(s) for s in sets]


def golden_neighbors(arr):
    return [sorted(int(j) for j in row if j >= 0) for row in arr]


def test_uniform_generator_matches_reference_functor():
    d = load("rng_uniform.npz")
    for seed in (1, 7, 12345):
        np.testing.assert_array_equal(fill_uniform(1000, 0.0, 38.5, 0, seed), d[f"uniform_seed{seed}"])
        np.testing.assert_array_equal(fill_uniform(1000, -0.5, 0.5, 3000, seed),
                                      d[f"uniform_seed{seed}_off"])


def test_normal_generator_statistics():
    v = fill_normal(20000, 0.0, 1.0, 1, 3)
    assert abs(v.mean()) < 0.03 and abs(v.std() - 1.0) < 0.03


def test_small_verlet_system():
    d = load("disk_n64_verlet.npz")
    o = make(d)
    assert_state(o, d, "setup")
    assert static_neighbors(o) == golden_neighbors(d["setup_neighbors"])
    o.nve_steps(1e-2, 200)
    assert_state(o, d, "nve200")
    o.fire_init(0.1, 1e-2)
    for _ in range(100):
        o.fire_step()
    assert_state(o, d, "fire100")
    fs = o.fire_state()
    np.testing.assert_array_equal(
        [fs["alpha"], fs["dt"], fs["n_good"], fs["n_bad"], fs["stopped"]], d["fire100_state"])


def test_cfg1_cell_system():
    d = load("disk_n1024_cell.npz")
    o = make(d)
    info = o.neighbor_info()
    assert info["n_cells_dim"] == int(d["n_cells_dim"]) and info["cap"] == int(d["cap"])
    ci, cs = o.cells()
    np.testing.assert_array_equal(ci, d["setup_cell_index"])
    np.testing.assert_array_equal(cs, d["setup_cell_start"])
    np.testing.assert_array_equal(o.get_current()["static_index"], d["setup_static_index"])
    assert_state(o, d, "setup")
    assert static_neighbors(o) == golden_neighbors(d["setup_neighbors"])
    np.testing.assert_array_equal(o.stress_tensor(), d["setup_stress"])
    assert o.contact_count() == float(d["setup_contacts"])
    o.nve_steps(1e-2, 500)
    assert_state(o, d, "nve500")
    assert tuple(o.num_rebuilds()) == tuple(d["nve500_rebuilds"])
    o.fire_init(0.1, 1e-2)
    for _ in range(300):
        o.fire_step()
    assert_state(o, d, "fire300")
    o.init_adam()
    for k in range(40):
        o.zero_force_and_pe()
        o.check_for_neighbor_update()
        o.calculate_forces()
        o.adam_step(k, 1e-3, 0.9, 0.999, 1e-8)
    assert_state(o, d, "adam40")


def test_fire_minimisation_to_reference_criteria():
    d = load("disk_n2048_fire_min.npz")
    o = make(d)
    steps, stopped = o.minimize_fire(0.1, 1e-2, 1e-16, 1e-16, 100000, 0.0)
    assert steps == int(d["steps"]) and stopped == int(d["stopped"])
    a = o.get_arrays()
    np.testing.assert_array_equal(a["x"], d["x"])
    np.testing.assert_array_equal(a["y"], d["y"])
    assert o.total_pe() / o.n == float(d["avg_pe"])
    assert o.pressure() == float(d["pressure"])


@pytest.mark.skipif(not reference_available(), reason="reference harness not built here")
def test_oracle_matches_reference_kernels_on_scaling_and_revert():
    d = load("disk_n1024_cell.npz")
    a, b = make(d, "oracle"), make(d, "reference")
    for o in (a, b):
        o.set_last_state()
        o.scale_to_packing_fraction(0.9)
        o.zero_force_and_pe()
        o.check_for_neighbor_update()
        o.calculate_forces()
        o.revert_to_last_state()
        o.scale_box(0.97)
        o.minimize_fire(0.1, 1e-2, 1e-16, 1e-16, 300, 0.0)
    ca, cb = a.get_current(), b.get_current()
    for k in ca:
        np.testing.assert_array_equal(ca[k], cb[k])
    assert a.box() == b.box()


def test_damped_nve_and_gradient_descent():
    """DampedNVE::step and GradDesc::step (src/integrator/damped_nve.cu:15-27,
    src/integrator/grad_desc.cu:11-17), with neighbour rebuilds along the way."""
    d = load("disk_n512_damped_gd.npz")
    o = make(d)
    o.damped_nve_steps(1e-2, 0.5, 300)
    assert_state(o, d, "damped300")
    assert list(o.num_rebuilds()) == list(d["damped300_rebuilds"])
    o.grad_desc_steps(1e-2, 200)
    assert_state(o, d, "gd200")
    assert list(o.num_rebuilds()) == list(d["gd200_rebuilds"])


def test_wall_forces_and_nve_wall_step():
    """calcWallInteraction / kernelCalcDiskWallForces and NVE::wall_step
    (include/particles/base/kernels.cuh:185-235, src/integrator/nve.cu:27-38)."""
    d = load("disk_n256_walls.npz")
    o = make(d)
    o.zero_force_and_pe()
    o.wall_forces()
    assert_state(o, d, "wall")
    o.nve_wall_steps(1e-2, 300)
    assert_state(o, d, "wallnve300")


def test_pair_and_hessian_dump():
    """kernelCalcDiskForceDistancePairs after the reference's fills: pair
    energies, forces, separations, ids, overlaps, angles and the pair / self
    Hessian blocks (src/particles/disk/kernels.cu:73-175)."""
    d = load("disk_n256_pairs.npz")
    o = make(d)
    o.nve_steps(1e-2, 50)
    assert o.neighbor_info()["cap"] == int(d["cap"])
    got = o.pair_dump()
    for k, v in got.items():
        np.testing.assert_array_equal(v, d[f"pairs_{k}"], err_msg=k)

"""CPU: the package's seeded initial states (dpcuda_gb300.init) reproduce the
reference's RandomUniform stream (include/functors.h:17-33) bit for bit: the
golden vectors made by the reference functor, and the oracle's generator."""
from pathlib import Path

import numpy as np

from dpcuda_gb300.init import disk_packing, random_uniform

G = Path(__file__).resolve().parent / "golden"


def test_random_uniform_matches_golden_vectors():
    d = dict(np.load(G / "rng_uniform.npz"))
    for seed in (1, 7, 12345):
        np.testing.assert_array_equal(random_uniform(1000, 0.0, 38.5, 0, seed), d[f"uniform_seed{seed}"])
        np.testing.assert_array_equal(random_uniform(1000, -0.5, 0.5, 3000, seed),
                                      d[f"uniform_seed{seed}_off"])


def test_random_uniform_matches_oracle_including_wraparound():
    from oracle.oracle import fill_uniform
    for n, lo, hi, off, seed in [(4096, 0.4, 0.6, 7 * 4096, 5), (100, 0.0, 1.0, 123456789, 2**32 - 1),
                                 (3000, -3.0, 2.0, 2**32 - 10, 77)]:
        np.testing.assert_array_equal(random_uniform(n, lo, hi, off, seed),
                                      fill_uniform(n, lo, hi, off, seed))


def test_disk_packing_matches_oracle():
    from oracle.oracle import disk_packing as oracle_packing
    a, b = disk_packing(2048, 0.86, 3), oracle_packing(2048, 0.86, 3)
    assert a["box"] == b["box"]
    for k in ("x", "y", "r", "m"):
        np.testing.assert_array_equal(a[k], b[k])


def test_bumpy_packing_matches_oracle():
    from oracle.oracle import bumpy_packing as oracle_bumpy
    from dpcuda_gb300.init import bumpy_packing
    a, b = bumpy_packing(256, 0.80, 5), oracle_bumpy(256, 0.80, 5)
    assert a["box"] == b["box"] and a["rv"] == b["rv"] and a["e_c"] == b["e_c"]
    for k in ("x", "y", "th", "r", "nvb"):
        np.testing.assert_array_equal(a[k], b[k])

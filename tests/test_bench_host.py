"""CPU: host logic of bench.py that every GPU run depends on.

* every execution form the ensemble autotuner can report has a form code in
  the bench (the headline sets the form the autotuner chose);
* the resident kernel's roofline: algorithmic bytes of a FIRE iteration
  (144 + 4k per disk) times the disk-iterations of the timed solves, over the
  region's time; the per-iteration time counts each batch's slowest system.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path[:0] = [str(ROOT), str(ROOT / "dpcuda-v2_gb300")]


def test_every_autotuner_form_has_a_bench_code():
    import bench
    from dpcuda_gb300 import ensemble
    for code, name in ensemble._FORM_NAMES.items():
        assert bench.FORM_CODES[name] == code


def test_resident_roofline_arithmetic():
    import bench
    k = 6.5
    results = [[{"fire_steps": 1000}] * 15 + [{"fire_steps": 3000}],
               [{"fire_steps": 2000}] * 16]
    total_ms, launches = 100.0, 4
    r = bench.resident_roofline(results, total_ms, launches, k, 6000.0, "test")
    per = 144 + 4 * k
    disk_iters = bench.N_PART * (15 * 1000 + 3000 + 16 * 2000)
    assert r["bytes_per_disk_iteration"] == pytest.approx(per)
    assert r["bytes_per_launch"] == pytest.approx(disk_iters * per / launches)
    assert r["launch_us"] == pytest.approx(total_ms * 1e3 / launches)
    achieved = disk_iters * per / (total_ms * 1e-3) / 1e9
    assert r["achieved"] == pytest.approx(achieved)
    assert r["frac"] == pytest.approx(achieved / 6000.0)
    assert r["us_per_iteration"] == pytest.approx(total_ms * 1e3 / (3000 + 2000))
    assert r["kernel"] == "e_res" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["traffic"] == pytest.approx(bench.E_RES_DRAM_PER_DISK * bench.BATCH * bench.N_PART)

"""Test configuration: the `gpu` marker and import paths.

-m "not gpu": oracle vs golden fixtures, host logic, C ABI exports (no GPU).
-m gpu:       CUDA path vs the oracle through the C ABI (needs a GB300).
"""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "dpcuda-v2_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")

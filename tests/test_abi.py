"""CPU: the C-ABI library builds for sm_103a, loads, and exports every entry
point that include/*.h declares (no compute calls: there is no GPU here)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(dpg_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "dpg_create" in names and "dpg_fire_minimize" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    from dpcuda_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(str(lib_path))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_abi():
    from dpcuda_gb300.lib import SIGNATURES
    missing = [n for n in declared_symbols() if n not in SIGNATURES]
    assert not missing, missing


def test_error_path_without_gpu_is_loud():
    """Creating a system must fail with a CUDA error, never fall back to CPU."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from dpcuda_gb300 import Disk, DpgError
    with pytest.raises(DpgError):
        Disk(16, 10.0)


def test_state_count_reads_the_reference_layout(tmp_path):
    """dpg_state_count is host-only: count the values of radii.dat written in the
    reference's StateLog format ("%.17e", one per line)."""
    import numpy as np
    from dpcuda_gb300 import Disk, DpgError
    r = np.linspace(0.5, 0.7, 37)
    (tmp_path / "radii.dat").write_text("".join(f"{v:.17e}\n" for v in r))
    assert Disk.stateCount(tmp_path) == 37
    with pytest.raises(DpgError):
        Disk.stateCount(tmp_path / "missing")


def test_bad_arguments_rejected_before_any_device_work():
    """dpg_create / dpg_ensemble_create check their arguments first, so bad
    sizes, boxes and precisions fail with DPG_ERR_ARG even without a GPU."""
    import ctypes as C
    from dpcuda_gb300.lib import EnsembleParams, Params, load_library
    DPG_ERR_ARG = 1  # include/dpg.h
    lib = load_library()
    h = C.c_void_p()
    for prm in (Params(0, 10.0, 10.0, 1.0, 2.0, 0, 0), Params(16, -1.0, 10.0, 1.0, 2.0, 0, 0),
                Params(16, 10.0, 10.0, 1.0, 2.0, 7, 0)):
        assert lib.dpg_create(C.byref(prm), None, C.byref(h)) == DPG_ERR_ARG
    n = (C.c_int64 * 1)(16)
    box = (C.c_double * 1)(10.0)
    for ep in (EnsembleParams(0, 1.0, 2.0, 1.7, 0.3, 0, 0, 0.0),
               EnsembleParams(1, 1.0, 2.0, -1.0, 0.3, 0, 0, 0.0),
               EnsembleParams(1, 1.0, 2.0, 1.7, 0.3, 5, 0, 0.0)):
        assert lib.dpg_ensemble_create(C.byref(ep), n, box, None, C.byref(h)) == DPG_ERR_ARG

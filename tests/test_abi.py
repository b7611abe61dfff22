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


def test_null_handles_rejected_for_rigid_and_ensemble_calls():
    """Every rigid-body and ensemble entry point added for the workflow pieces
    checks its handle first and returns DPG_ERR_ARG without device work."""
    import ctypes as C
    from dpcuda_gb300.lib import load_library
    DPG_ERR_ARG = 1
    lib = load_library()
    calls = [
        ("dpg_bumpy_adam_init", ()), ("dpg_bumpy_adam_step", (C.c_int64(0), C.c_double(1e-3),
                                      C.c_double(0.9), C.c_double(0.999), C.c_double(1e-8))),
        ("dpg_bumpy_damped_forces", (C.c_double(0.1),)),
        ("dpg_bumpy_damped_nve_steps", (C.c_double(1e-3), C.c_double(0.1), C.c_int64(1))),
        ("dpg_bumpy_wall_forces", (C.c_int(0),)),
        ("dpg_bumpy_nve_wall_steps", (C.c_double(1e-3), C.c_int64(1))),
        ("dpg_bumpy_grad_desc_step", (C.c_double(1e-3),)),
        ("dpg_bumpy_grad_desc_steps", (C.c_double(1e-3), C.c_int64(1))),
        ("dpg_bumpy_stress", (None, None, None)),
        ("dpg_bumpy_contacts", (None, None, None, None)),
        ("dpg_bumpy_save_state", ()), ("dpg_bumpy_restore_state", ()),
        ("dpg_bumpy_pair_dump", (None, None, None, None, C.c_int(0))),
        ("dpg_bumpy_counts", (None, None)),
        ("dpg_bumpy_get_static", (None, None, None, None, None)),
        ("dpg_bumpy_set_box", (C.c_double(10.0), C.c_double(10.0))),
        ("dpg_bumpy_packing_fraction", (None,)),
        ("dpg_bumpy_write_state", (b"/nonexistent", C.c_int64(-1))),
        ("dpg_bumpy_read_state", (b"/nonexistent",)),
        ("dpg_ensemble_set_form", (C.c_int(1), C.c_int(0))),
        ("dpg_set_force_group", (C.c_int(2),)),
        ("dpg_autotune_force_group", (C.c_int(10), None, None)),
        ("dpg_ensemble_autotune", (None, C.c_int(10), None)),
    ]
    for name, args in calls:
        assert getattr(lib, name)(None, *args) == DPG_ERR_ARG, name


def test_bumpy_state_count_reads_the_reference_layout(tmp_path):
    """dpg_bumpy_state_count is host-only: bodies from radii.dat, vertices from
    the "x<TAB>y" lines of vertex_positions.dat."""
    import numpy as np
    from dpcuda_gb300.bumpy import bumpyStateCount
    (tmp_path / "radii.dat").write_text("".join(f"{v:.17e}\n" for v in np.full(5, 0.5)))
    (tmp_path / "vertex_positions.dat").write_text(
        "".join(f"{a:.17e}\t{b:.17e}\n" for a, b in np.random.default_rng(1).random((83, 2))))
    assert bumpyStateCount(tmp_path) == (5, 83)


def test_header_is_plain_c_and_links_every_symbol(tmp_path):
    """include/dpg.h compiles as C99 (no C++ types in the signatures), and a C
    program that takes the address of every declared entry point links
    against the built library (the C linkage a cgo / ctypes / JNI stub binds)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no C compiler")
    from dpcuda_gb300 import build
    lib = build.build()
    names = declared_symbols()
    src = ['#include "dpg.h"', "#include <stdio.h>", "int main(void) {", "    void *p[] = {"]
    src += [f"        (void *)&{n}," for n in names]
    src += ["    };", '    printf("%d\\n", (int)(sizeof p / sizeof p[0]));', "    return 0;", "}"]
    c = tmp_path / "abi_check.c"
    c.write_text("\n".join(src) + "\n")
    exe = tmp_path / "abi_check"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-pedantic-errors", "-Wno-pedantic",
                    "-I", str(ROOT / "include"), str(c), "-o", str(exe),
                    "-L", str(lib.parent), "-ldpg", f"-Wl,-rpath,{lib.parent}"],
                   check=True, capture_output=True)
    assert exe.exists()

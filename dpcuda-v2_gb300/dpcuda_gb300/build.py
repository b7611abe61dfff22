"""Builds the in-tree CUDA library ``_build/libdpg.so`` for sm_103a.

The library is plain nvcc output (no torch extension): one translation unit
per precision form, linked into one shared object whose entry points are the
C ABI declared in ``include/dpg.h``.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # dpcuda-v2_gb300/
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
BUILD = PKG_ROOT / "_build"
LIB = BUILD / "libdpg.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(REPO_ROOT / "include")]

# (source, extra flags).  The FP64 drop-in is compiled without FMA contraction
# so its arithmetic is the reference's, operation for operation.
UNITS = [
    ("disk_system.cu", ["--fmad=false"]),
    ("bumpy_system.cu", ["--fmad=false"]),
    ("ensemble_system.cu", []),
    ("noalloc.cu", ["--fmad=false"]),
    ("peaks.cu", []),
    ("jam.cpp", []),
    ("state_io.cpp", []),
]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + \
        sorted(CSRC.glob("*.cpp")) + \
        [REPO_ROOT / "include" / "dpg.h"]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in sources() if p.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    units = [(CSRC / src, flags) for src, flags in UNITS if (CSRC / src).exists()]

    def compile_one(item):
        src, flags = item
        obj = BUILD / (src.stem + ".o")
        cmd = [nvcc, *ARCH, *COMMON, *flags, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, len(units))) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = BUILD / "libdpg.so.tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *[str(o) for o in objs], "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))

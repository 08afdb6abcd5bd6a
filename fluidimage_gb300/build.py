"""Build ``libfluidimage_gb300.so`` in-tree from ``csrc/*.cu`` for sm_103a.

Each translation unit is compiled in parallel with nvcc, then linked into one
shared library exporting the C ABI of ``include/fluidimage_gb300.h``.  The build
is skipped when the library is newer than every source and header.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIBNAME = "libfluidimage_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fluidimage_gb300")


def library_path() -> Path:
    return LIBDIR / LIBNAME


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _deps():
    return _sources() + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "fluidimage_gb300.h"]


def up_to_date() -> bool:
    lib = library_path()
    if not lib.exists():
        return False
    mtime = lib.stat().st_mtime
    return all(p.stat().st_mtime <= mtime for p in _deps())


def build(force: bool = False, verbose: bool = False) -> Path:
    lib = library_path()
    if not force and up_to_date():
        return lib
    nvcc = nvcc_path()
    objdir = LIBDIR / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]

    def compile_one(src: Path) -> Path:
        obj = objdir / (src.stem + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *inc, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as pool:
        objs = list(pool.map(compile_one, _sources()))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "--cudart", "static", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose=True)
    print(path)

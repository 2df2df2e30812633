"""In-tree build of the CUDA engine: fasticgn_gb300/libdic.so for sm_103a.

One translation unit (csrc/dic_engine.cu, which includes csrc/dic_kernels.cuh) compiled by
nvcc with one -gencode, so a build takes seconds on any host that has nvcc; no GPU needed.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
LIB = PKG / "libdic.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 DIC engine needs the CUDA toolkit to build")


def sources():
    return [CSRC / "dic_engine.cu", CSRC / "dic_kernels.cuh", INCLUDE / "dic.h"]


def build_lib(force: bool = False, verbose: bool = False, extra=()) -> Path:
    newest = max(p.stat().st_mtime for p in sources())
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_name(f"libdic.so.tmp{os.getpid()}")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-I", str(INCLUDE), str(CSRC / "dic_engine.cu"), "-o", str(tmp), *extra]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_lib(force="--force" in sys.argv, verbose=True))

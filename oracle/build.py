"""Build recipe for the oracle (test infrastructure, not the product).

Compiles oracle/dic_oracle.cpp, the CPU restatement of OpenCorr's FFTCC2D / ICGN2D1 path,
into oracle/libdic_oracle.so with g++ and OpenMP.  FP contraction is disabled so the x86_64
build container and the aarch64 GPU host produce identical bits.

The reference's own CPU implementation cannot be compiled here: its sources include Eigen,
OpenCV and FFTW headers and none of the three is installed.  What does compile from the
reference tree is the xxHash header it vendors (third_party/xxhash/xxhash.h, header-only):
build_xxh3_ref() compiles oracle/xxh3_check.c against it where it lies into
oracle/_ref/xxh3_ref, the checker for the output ledger's XXH3-128 (only where the
reference tree is present; the golden digests it produced are committed under tests/golden).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "dic_oracle.cpp"
LIB = HERE / "libdic_oracle.so"


def build_oracle(force: bool = False, verbose: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           str(SRC), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


REF_ROOT = Path("/root/reference")
REF_DIR = HERE / "_ref"


def build_xxh3_ref(force: bool = False, verbose: bool = False) -> Path | None:
    """oracle/_ref/xxh3_ref from the reference's vendored xxhash.h; None without the tree."""
    header_dir = REF_ROOT / "third_party" / "xxhash"
    src = HERE / "xxh3_check.c"
    exe = REF_DIR / "xxh3_ref"
    if not (header_dir / "xxhash.h").exists():
        return exe if exe.exists() else None
    if not force and exe.exists() and exe.stat().st_mtime >= src.stat().st_mtime:
        return exe
    REF_DIR.mkdir(exist_ok=True)
    tmp = exe.with_name(f"xxh3_ref.tmp{os.getpid()}")
    cmd = ["gcc", "-O2", "-I", str(header_dir), str(src), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, exe)
    return exe


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv, verbose=True))
    print(build_xxh3_ref(force="--force" in sys.argv, verbose=True))

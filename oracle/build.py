"""Build recipe for the oracle (test infrastructure, not the product).

Compiles oracle/dic_oracle.cpp, the CPU restatement of OpenCorr's FFTCC2D / ICGN2D1 path,
into oracle/libdic_oracle.so with g++ and OpenMP.  FP contraction is disabled so the x86_64
build container and the aarch64 GPU host produce identical bits.

The reference's own CPU implementation cannot be compiled here: its sources include Eigen,
OpenCV and FFTW headers and none of the three is installed.  What does compile from the
reference tree is the xxHash header it vendors (third_party/xxhash/xxhash.h, header-only):
build_xxh3_ref() compiles oracle/xxh3_check.c against it where it lies into
oracle/_ref/xxh3_ref, the checker for the output ledger's XXH3-128 (only where a reference
checkout is named; the golden digests it produced are committed under tests/golden).

The checkout is named by the --reference argument or the DIC_REFERENCE environment variable:

    DIC_REFERENCE=/path/to/FastICGN python oracle/build.py
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


REF_DIR = HERE / "_ref"


def reference_root(reference: str | os.PathLike | None = None) -> Path | None:
    """The reference checkout: the argument, else $DIC_REFERENCE, else None."""
    root = reference or os.environ.get("DIC_REFERENCE")
    return Path(root) if root else None


def build_xxh3_ref(force: bool = False, verbose: bool = False, reference=None) -> Path | None:
    """oracle/_ref/xxh3_ref from the reference's vendored xxhash.h; None without a checkout."""
    exe = REF_DIR / "xxh3_ref"
    root = reference_root(reference)
    if root is None:
        return exe if exe.exists() else None
    header_dir = root / "third_party" / "xxhash"
    src = HERE / "xxh3_check.c"
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
    import argparse
    ap = argparse.ArgumentParser(description="build the oracle (and the xxHash checker from a reference checkout)")
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--reference", default=None, help="reference checkout (default: $DIC_REFERENCE)")
    a = ap.parse_args()
    print(build_oracle(force=a.force, verbose=True))
    print(build_xxh3_ref(force=a.force, verbose=True, reference=a.reference))

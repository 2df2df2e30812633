"""Build recipe for the oracle (test infrastructure, not the product).

Compiles oracle/dic_oracle.cpp, the CPU restatement of OpenCorr's FFTCC2D / ICGN2D1 path,
into oracle/libdic_oracle.so with g++ and OpenMP.  FP contraction is disabled so the x86_64
build container and the aarch64 GPU host produce identical bits.

The reference's own CPU implementation cannot be compiled here: its sources include Eigen,
OpenCV and FFTW headers and none of the three is installed, so there is no oracle/_ref.
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


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv, verbose=True))

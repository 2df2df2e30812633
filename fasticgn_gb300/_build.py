"""In-tree build of the CUDA engine (fasticgn_gb300/libdic.so for sm_103a) and of the
command line over it (fasticgn_gb300/opencorr_cli_gb300).

The engine is one translation unit (csrc/dic_engine.cu, which includes the csrc/*.cuh
kernels) compiled by nvcc with one -gencode, so a build takes seconds on any host that has
nvcc; no GPU needed.  The command line is plain C++17 (g++) linked against libdic.so.
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


CLI_DIR = PKG / "cli"
CLI = PKG / "opencorr_cli_gb300"


def sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "dic.h"]


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


def _git(*args) -> str | None:
    try:
        out = subprocess.run(["git", *args], cwd=PKG.parent, capture_output=True, text=True, timeout=10)
    except (OSError, subprocess.SubprocessError):
        return None
    return out.stdout.strip() if out.returncode == 0 else None


def build_cli(force: bool = False, verbose: bool = False) -> Path:
    """The command line (cli/*.cpp), with the commit and build time it was built from."""
    lib = build_lib(verbose=verbose)
    srcs = sorted(CLI_DIR.glob("*.cpp")) + sorted(CLI_DIR.glob("*.h"))
    newest = max([p.stat().st_mtime for p in srcs] + [lib.stat().st_mtime, (INCLUDE / "dic.h").stat().st_mtime])
    if not force and CLI.exists() and CLI.stat().st_mtime >= newest:
        return CLI
    import datetime
    head = _git("rev-parse", "--short=12", "HEAD")
    status = _git("status", "--porcelain", "--untracked-files=no")
    dirty = "" if status is None else ("1" if status else "0")
    date = datetime.datetime.now(datetime.timezone.utc).strftime("%Y-%m-%dT%H:%M:%SZ")
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("a C++17 compiler (g++) is needed for the command line")
    tmp = CLI.with_name(f"{CLI.name}.tmp{os.getpid()}")
    cmd = [cxx, "-O3", "-std=c++17", "-Wall", "-I", str(INCLUDE),
           f'-DDIC_CLI_GIT_HASH="{head or "unknown"}"', f'-DDIC_CLI_BUILD_DATE="{date}"',
           f'-DDIC_CLI_GIT_DIRTY="{dirty}"',
           *[str(p) for p in sorted(CLI_DIR.glob("*.cpp"))], "-o", str(tmp),
           "-L", str(PKG), "-ldic", "-Wl,-rpath,$ORIGIN", "-pthread"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    print(build_lib(force="--force" in sys.argv, verbose=True))
    print(build_cli(force="--force" in sys.argv, verbose=True))

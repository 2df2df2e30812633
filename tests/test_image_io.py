"""The command line's image decoder on the CPU: decoding a sequence of PGM and TIFF files of
different sizes and depths while reusing the previous frame's buffers (the frame loop's
path) gives what a fresh decode gives, and both agree with the pixels written."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import cli_files as F

ROOT = Path(__file__).resolve().parent.parent
CLI = ROOT / "fasticgn_gb300" / "cli"


def fnv(img: np.ndarray) -> int:
    h = 1469598103934665603
    for v in img.ravel().tolist():
        h = ((h ^ int(v)) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def test_reused_buffers_decode_like_fresh(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    exe = tmp_path / "image_io_main"
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", str(CLI), str(ROOT / "tests" / "image_io_main.cpp"),
                    str(CLI / "image_io.cpp"), "-o", str(exe)], check=True)
    rng = np.random.default_rng(3)
    cases = [("a.pgm", rng.integers(0, 4096, (40, 56)).astype(np.uint16), "pgm", 4095),
             ("b.pgm", rng.integers(0, 256, (24, 30)).astype(np.uint8), "pgm", 255),      # 8-bit after 16-bit
             ("c.pgm", rng.integers(0, 65536, (64, 72)).astype(np.uint16), "pgm", 65535),  # larger again
             ("d.tif", rng.integers(0, 65536, (16, 20)).astype(np.uint16), "tif", None),   # smaller, TIFF
             ("e.pgm", rng.integers(0, 4096, (40, 56)).astype(np.uint16), "pgm", 4095)]
    for name, img, kind, maxval in cases:
        if kind == "pgm":
            F.write_pgm(tmp_path / name, img, maxval=maxval)
        else:
            F.write_tiff(tmp_path / name, img)
    out = subprocess.run([str(exe), *[str(tmp_path / c[0]) for c in cases]], check=True, capture_output=True,
                         text=True).stdout.splitlines()
    assert len(out) == 2 * len(cases)
    for k, (name, img, _, _) in enumerate(cases):
        fresh, reused = out[2 * k].split(), out[2 * k + 1].split()
        assert fresh[0] == "fresh" and reused[0] == "reused"
        assert fresh[2:] == reused[2:], (name, fresh, reused)
        w, h, bits, lo, hi, cs = fresh[2:]
        assert (int(h), int(w)) == img.shape and int(bits) == (8 if img.dtype == np.uint8 else 16)
        assert float(lo) == img.min() and float(hi) == img.max() and int(cs) == fnv(img), name

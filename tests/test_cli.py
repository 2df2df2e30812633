"""Command line without a GPU: argv surface and strict parsing, status line, tar list
errors and image decoding (the smoke/test_cli_interface.py kind of checks of the
reference, restated for this binary).  Nothing here creates an engine."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import cli_files as F

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def cli():
    sys.path.insert(0, str(ROOT))
    from fasticgn_gb300 import _build
    return _build.build_cli()


def test_version_and_help(cli):
    out = subprocess.run([str(cli), "--version"], capture_output=True, text=True, check=True).stdout
    keys = dict(ln.partition("=")[::2] for ln in out.splitlines() if "=" in ln)
    # the pipeline's --version probe reads git_hash= and build_date= (dic_pipeline.py:1222-1250)
    assert keys["name"] == "opencorr_cli_gb300" and keys["git_hash"] and keys["build_date"]
    assert keys["backend"] == "cuda"
    h = subprocess.run([str(cli), "--help"], capture_output=True, text=True)
    assert h.returncode == 0 and "--multi-frame" in h.stdout and not h.stdout.strip().startswith("{")


@pytest.mark.parametrize("args,needle", [
    (["--multi-frame", "--ref", "r.pgm", "--tar-list", "l.txt", "--output-dir", "o", "7"], "positional"),
    (["--multi-frame", "--ref", "r.pgm", "--tar-list", "l.txt", "--output-dir", "o", "7", "2", "--max-iter", "0"],
     "--max-iter out of range"),
    (["--multi-frame", "--ref", "r.pgm", "--tar-list", "l.txt", "--output-dir", "o", "7", "2", "--bogus"],
     "unknown option: --bogus"),
    (["--multi-frame", "--ref", "r.pgm", "--tar-list", "l.txt", "--output-dir", "o", "7", "2", "--subset-size", "15"],
     "conflicts"),
    (["--multi-frame", "--ref", "r.pgm", "--tar-list", "l.txt", "--output-dir", "o", "7", "2", "--subset-size", "14"],
     "odd subset SIZE"),
    (["--multi-frame", "--ref", "r.pgm", "--tar-list", "l.txt", "--output-dir", "o", "7", "2", "--input-align", "left"],
     "--input-align is only meaningful"),
    (["--multi-frame", "--ref", "r.pgm", "--tar-list", "l.txt", "--output-dir", "o", "7", "2", "--conv-threshold", "-1"],
     "finite positive"),
    (["--multi-frame", "--ref", "r.pgm", "--tar-list", "l.txt", "--output-dir", "o", "7", "2", "--dual-gpu"],
     "not available"),
    (["--multi-frame", "--ref", "r.pgm", "--tar-list", "l.txt", "--output-dir", "o", "0", "2"], "subset_radius out of range"),
    (["a.pgm", "b.pgm", "7", "2"], "positional"),
])
def test_rejected_command_lines(cli, tmp_path, args, needle):
    rc, status, err = F.run_cli(cli, args, cwd=tmp_path)
    assert rc == 1
    assert status["status"] == "error" and status["exit_code"] == 1 and needle in status["error"], status
    assert any(ln.startswith("Error:") for ln in err.splitlines())
    assert status["schema"] == "fasticgn.run-status/1" and status["tool"] == "opencorr_cli_gb300"


def verify_only(cli, *args):
    p = subprocess.run([str(cli), "--verify-only", *map(str, args)], capture_output=True, text=True)
    lines = p.stdout.strip().splitlines()
    assert len(lines) == 1, p.stdout
    return p.returncode, json.loads(lines[0]), p.stderr


def test_verify_only_without_a_run(cli, tmp_path):
    """--verify-only answers with one JSON verdict (schema fasticgn.verify-only/1) for every
    invocation and exits 0 only for a complete run."""
    rc, v, err = verify_only(cli, tmp_path / "nope")
    assert rc == 1 and v["schema"] == "fasticgn.verify-only/1" and v["status"] == "not_found" and v["exit_code"] == 1
    rc, v, _ = verify_only(cli, tmp_path)
    assert rc == 1 and v["status"] == "not_a_run" and v["complete"] is False
    rc, v, err = verify_only(cli)
    assert rc == 1 and v["status"] == "error" and v["output_dir"] is None and "exactly one argument" in v["problems"][0]
    assert err.startswith("Error:")
    rc, v, _ = verify_only(cli, tmp_path, tmp_path)
    assert rc == 1 and v["status"] == "error"
    (tmp_path / "d" / ".opencorr-state").mkdir(parents=True)
    (tmp_path / "d" / ".opencorr-state" / "contract.json").write_text('{"targets": []')
    rc, v, _ = verify_only(cli, tmp_path / "d")
    assert rc == 1 and v["status"] == "damaged" and "not a usable run contract" in v["problems"][0]
    assert v["tool"] == "opencorr_cli_gb300"


def test_multi_frame_ledger_refusals_before_the_gpu(cli, tmp_path):
    """A dedicated output directory: a stray output file or an unknown entry stops a new run
    before the engine is created (checked on the CPU; the GPU tests cover runs)."""
    ref = (np.arange(64 * 48) % 251).astype(np.uint8).reshape(48, 64)
    F.write_pgm(tmp_path / "ref.pgm", ref)
    F.write_pgm(tmp_path / "t0.pgm", ref)
    (tmp_path / "list.txt").write_text(f"{tmp_path / 't0.pgm'} frame_000000.csv\n")
    out = tmp_path / "out"
    out.mkdir()
    (out / "frame_000000.csv").write_text("x,y\n")
    base = ["--multi-frame", "--ref", tmp_path / "ref.pgm", "--tar-list", tmp_path / "list.txt", "--output-dir", out, "7", "4"]
    rc, status, err = F.run_cli(cli, base)
    assert rc == 1 and "existing output has no verified run record" in status["error"], status
    (out / "frame_000000.csv").unlink()
    (out / "notes.txt").write_text("n")
    rc, status, err = F.run_cli(cli, base)
    assert rc == 1 and "untracked entry in output directory" in status["error"], status
    assert not (out / ".opencorr-state").exists()        # a refused run records nothing


def test_tar_list_errors(cli, tmp_path):
    ref = (np.arange(64 * 48) % 251).astype(np.uint8).reshape(48, 64)
    F.write_pgm(tmp_path / "ref.pgm", ref)
    (tmp_path / "bad.txt").write_text(f"{tmp_path / 'ref.pgm'}\n")
    rc, status, _ = F.run_cli(cli, ["--multi-frame", "--ref", tmp_path / "ref.pgm", "--tar-list", tmp_path / "bad.txt",
                                    "--output-dir", tmp_path / "out", "7", "4"])
    assert rc == 1 and "invalid tar list line" in status["error"]
    (tmp_path / "empty.txt").write_text("\n\n")
    rc, status, _ = F.run_cli(cli, ["--multi-frame", "--ref", tmp_path / "ref.pgm", "--tar-list", tmp_path / "empty.txt",
                                    "--output-dir", tmp_path / "out", "7", "4"])
    assert rc == 1 and "tar list is empty" in status["error"]


def test_image_errors_before_compute(cli, tmp_path):
    a = np.zeros((40, 50), np.uint8)
    F.write_pgm(tmp_path / "a.pgm", a)
    F.write_pgm(tmp_path / "b.pgm", np.zeros((41, 50), np.uint8))
    (tmp_path / "c.png").write_bytes(b"\x89PNG\r\n\x1a\n")
    rc, status, _ = F.run_cli(cli, [tmp_path / "a.pgm", tmp_path / "b.pgm", "7", "4", tmp_path / "o.csv"])
    assert rc == 1 and "sizes differ" in status["error"]
    rc, status, _ = F.run_cli(cli, [tmp_path / "a.pgm", tmp_path / "c.png", "7", "4", tmp_path / "o.csv"])
    assert rc == 1 and "unsupported image format" in status["error"]
    F.write_pgm(tmp_path / "d.pgm", np.full((40, 50), 4096 + 7, np.uint16))
    rc, status, _ = F.run_cli(cli, [tmp_path / "d.pgm", tmp_path / "d.pgm", "7", "4", tmp_path / "o.csv",
                                    "--input-depth", "12", "--input-align", "right"])
    assert rc == 1 and "above 4095" in status["error"]


DECODE_HARNESS = r"""
#include "image_io.h"
#include <cstdio>
int main(int argc, char** argv) {
  dic_cli::Image img = dic_cli::read_image(argv[1]);
  std::FILE* f = std::fopen(argv[2], "wb");
  std::fprintf(f, "%d %d %d\n", img.width, img.height, img.bits);
  if (img.bits == 8) std::fwrite(img.u8.data(), 1, img.u8.size(), f);
  else std::fwrite(img.u16.data(), 2, img.u16.size(), f);
  std::fclose(f);
  return 0;
}
"""


@pytest.fixture(scope="module")
def decoder(tmp_path_factory):
    d = tmp_path_factory.mktemp("dec")
    (d / "h.cpp").write_text(DECODE_HARNESS)
    exe = d / "dec"
    cli_dir = ROOT / "fasticgn_gb300" / "cli"
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", str(cli_dir), str(d / "h.cpp"), str(cli_dir / "image_io.cpp"),
                    "-o", str(exe)], check=True)
    return exe


def _decode(exe, path, out):
    subprocess.run([str(exe), str(path), str(out)], check=True)
    raw = Path(out).read_bytes()
    head, _, body = raw.partition(b"\n")
    w, h, bits = map(int, head.split())
    return np.frombuffer(body, dtype=np.uint8 if bits == 8 else np.uint16).reshape(h, w)


@pytest.mark.parametrize("kind", ["pgm8", "pgm16", "pgm_ascii", "tiff8_le", "tiff16_le", "tiff16_be"])
def test_decoders(decoder, tmp_path, kind):
    rng = np.random.default_rng(3)
    img8 = rng.integers(0, 256, (37, 53), dtype=np.uint8)
    img16 = rng.integers(0, 4096, (37, 53), dtype=np.uint16)
    p = tmp_path / "img"
    if kind == "pgm8":
        F.write_pgm(p, img8); want = img8
    elif kind == "pgm16":
        F.write_pgm(p, img16, maxval=4095); want = img16
    elif kind == "pgm_ascii":
        F.write_pgm(p, img8, ascii_=True); want = img8
    elif kind == "tiff8_le":
        F.write_tiff(p, img8); want = img8
    elif kind == "tiff16_le":
        F.write_tiff(p, img16); want = img16
    else:
        F.write_tiff(p, img16, big_endian=True); want = img16
    got = _decode(decoder, p, tmp_path / "out")
    np.testing.assert_array_equal(got, want)

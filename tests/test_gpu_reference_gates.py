"""The reference's own consumers against opencorr_cli_gb300, the drop-in for its
opencorr_cli_cuda_mvp: its binary-driven gates (smoke/run_frame_fallback_gate.py,
run_oob_rejection_gate.py, run_zero_texture_gate.py, run_subpixel_accuracy_gate.py, each
given --binary) and the pipeline's reader of the raw output (pipeline/fasticgn_io.py:
read_manifest / iter_frames / read_raw_frame, read_ledger and run_status).

These scripts live in a reference checkout, named by $DIC_REFERENCE; nothing of the
reference is copied into this repository, and without a checkout the tests skip.
"""
import importlib.util
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
CLI = ROOT / "fasticgn_gb300" / "opencorr_cli_gb300"


@pytest.fixture(scope="module")
def reference():
    root = os.environ.get("DIC_REFERENCE")
    if not root or not (Path(root) / "smoke").is_dir() or not (Path(root) / "pipeline").is_dir():
        pytest.skip("no reference checkout named by $DIC_REFERENCE")
    return Path(root).resolve()


@pytest.fixture(scope="module")
def cli(dic):
    from fasticgn_gb300 import _build
    return _build.build_cli()


ZERO_TEXTURE_CODE = pytest.mark.xfail(
    strict=True,
    reason="the gate expects -3 for zero-texture subsets from a CUDA build (the reference CUDA kernel's extra "
           "reference-side rejection); this engine follows the CPU path, the parity oracle, which gives -5 "
           "(tests/test_gpu_parity.py::test_zero_texture_cpu_rule)")


@pytest.mark.parametrize("gate", ["run_frame_fallback_gate.py", "run_oob_rejection_gate.py",
                                  pytest.param("run_zero_texture_gate.py", marks=ZERO_TEXTURE_CODE),
                                  "run_subpixel_accuracy_gate.py"])
def test_reference_gate_passes(reference, cli, gate, tmp_path):
    script = reference / "smoke" / gate
    p = subprocess.run([sys.executable, str(script), "--binary", str(cli), "--work-dir", str(tmp_path / "evidence")],
                       capture_output=True, text=True, timeout=1800, cwd=str(reference / "smoke"))
    assert p.returncode == 0, f"{gate} rc {p.returncode}\n{p.stdout[-3000:]}\n{p.stderr[-2000:]}"


def load_reader(reference):
    spec = importlib.util.spec_from_file_location("fasticgn_io_reference", reference / "pipeline" / "fasticgn_io.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_pipeline_reader_reads_the_raw_output(reference, cli, dic, tmp_path):
    """A 12-bit multi-frame run of the command line, read by the pipeline's own reader: the
    manifest passes its checks, every frame's records equal the engine's results for the
    same frames (x, y, u, v, ux, uy, vx, vy, zncc), and run_status calls the directory
    complete."""
    io = load_reader(reference)
    from fasticgn_gb300 import speckle
    ref, frames = speckle.stream_frames(width=256, height=224, frames=200, which=[10, 11, 12, 13])
    radius, step = 12, 6

    def pgm(path, img):
        h, w = img.shape
        path.write_bytes(f"P5\n{w} {h}\n4095\n".encode() + img.astype(">u2").tobytes())

    pgm(tmp_path / "ref.pgm", ref)
    lines = []
    for k, (_, tar, _) in enumerate(frames):
        pgm(tmp_path / f"tar_{k}.pgm", tar)
        lines.append(f"{tmp_path / f'tar_{k}.pgm'} frame_{k:06d}.bin")
    (tmp_path / "list.txt").write_text("\n".join(lines) + "\n")
    out = tmp_path / "out"
    p = subprocess.run([str(cli), "--multi-frame", "--ref", str(tmp_path / "ref.pgm"), "--tar-list",
                        str(tmp_path / "list.txt"), "--output-dir", str(out), str(radius), str(step),
                        "--input-depth", "12", "--output-format", "raw", "--gpu-device", "0"],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]

    manifest = io.read_manifest(io.manifest_path(out))
    got = list(io.iter_frames(io.manifest_path(out)))
    assert len(got) == len(frames)
    tmpl = dic.grid_queue(256, 224, radius, step)
    e = dic.Engine(radius)
    e.set_ref(ref)
    e.sequence_begin(tmpl)
    for (entry, records), (_, tar, _) in zip(got, frames):
        want = np.zeros_like(tmpl)
        e.sequence_frame(tar, want)
        assert records.shape[0] == len(tmpl)
        assert np.array_equal(records["x"], tmpl["x"].astype(np.int32))
        assert np.array_equal(records["y"], tmpl["y"].astype(np.int32))
        for name in ("u", "v", "ux", "uy", "vx", "vy", "zncc"):
            assert np.array_equal(records[name].view(np.uint32), want[name].view(np.uint32)), (entry, name)
    e.close()
    frames_in_dir = [path.name for path, _ in io.iter_frame_dir(out)]
    assert frames_in_dir == [f"frame_{k:06d}.bin" for k in range(len(frames))]
    assert io.engine_metadata(manifest), "the manifest carries an engine block"
    ledger = io.read_ledger(out)
    assert ledger["present"] and "contract.json" in ledger and "complete.json" in ledger
    status = io.run_status(out)
    assert status["verdict"] == "complete" and status["complete"], json.dumps(status)[:2000]
    assert status["frames"]["expected"] == len(frames) and status["frames"]["present"] == len(frames)

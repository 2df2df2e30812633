"""The command line end to end on the GPU: multi-frame raw runs (records + manifest as the
pipeline reads them), CSV output, single-frame mode, 12-bit input handling, --line and the
output filters.  Records are checked bit for bit against the engine's own sequence API on
the same inputs, and the solution against the synthetic truth."""
import json
import subprocess

import numpy as np
import pytest

import cli_files as F
import dic_checks as C

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cli(dic):
    from fasticgn_gb300 import _build
    return _build.build_cli()


@pytest.fixture(scope="module")
def stream12(tmp_path_factory):
    """Six 12-bit frames of the sine/strain stream, written as 16-bit PGM (maxval 4095)."""
    from fasticgn_gb300 import speckle
    d = tmp_path_factory.mktemp("stream12")
    ref, frames = speckle.stream_frames(width=256, height=224, frames=200, which=[0, 1, 2, 3, 4, 5])
    F.write_pgm(d / "ref.pgm", ref, maxval=4095)
    lines = []
    for k, tar, _ in frames:
        F.write_pgm(d / f"tar {k:03d}.pgm", tar, maxval=4095)      # a space in the path, as camera exports have
        lines.append(f"{d / f'tar {k:03d}.pgm'} frame_{k:06d}.csv")
    (d / "tar_list.txt").write_text("\n".join(lines) + "\n")
    return d, ref, [f[1] for f in frames], [f[2] for f in frames]


def engine_sequence(dic, ref, tars, radius, step, lines=None, skip=True, poi_fallback=True):
    tmpl = dic.grid_queue(ref.shape[1], ref.shape[0], radius, step, lines=lines)
    e = dic.Engine(radius)
    e.set_ref(ref)
    e.sequence_begin(tmpl, skip_fftcc=skip, poi_fallback=poi_fallback)
    out = []
    for tar in tars:
        res = np.zeros_like(tmpl)
        rep = e.sequence_frame(tar, res)
        out.append((res, rep))
    e.close()
    return out


def test_multi_frame_raw_matches_engine(dic, cli, stream12, tmp_path):
    d, ref, tars, fields = stream12
    out = tmp_path / "out"
    rc, status, err = F.run_cli(cli, ["--multi-frame", "--ref", d / "ref.pgm", "--tar-list", d / "tar_list.txt",
                                      "--output-dir", out, "12", "8", "--input-depth", "12", "--output-format", "raw",
                                      "--gpu-device", "0"])
    assert rc == 0, err
    assert status["status"] == "ok" and status["frames_processed"] == 6 and status["mode"] == "multi-frame"
    assert status["totals"]["skip_fftcc_frames"] == 5
    assert "Reference input: source_depth=CV_16U" in err and "effective_depth=12" in err
    m = F.read_manifest(out / "manifest.opencorr-raw.json")
    assert m["subset_radius"] == 12 and m["grid_space"] == 8 and m["engine"]["oob_policy"] == "geometric-v1"
    assert m["engine"]["frame_fallback_policy"] == "per-poi-merge-v1" and m["input_image"]["depth"] == "12"
    assert [f["file"] for f in m["frames"]] == [f"frame_{k:06d}.bin" for k in range(6)]
    assert [f["output_name"] for f in m["frames"]] == [f"frame_{k:06d}.csv" for k in range(6)]
    want = engine_sequence(dic, ref, tars, 12, 8)
    for k, ((entry, rec), (res, rep)) in enumerate(zip(F.iter_frames(out / "manifest.opencorr-raw.json"), want)):
        assert np.array_equal(rec["x"], res["x"].astype(np.int32)) and np.array_equal(rec["y"], res["y"].astype(np.int32))
        for name in ("u", "v", "ux", "uy", "vx", "vy", "zncc"):
            np.testing.assert_array_equal(rec[name], res[name], err_msg=f"frame {k} {name}")
        assert entry["skip_fftcc_used"] == (k > 0) and entry["fallback_used"] is False
        assert entry["valid_ratio"] == pytest.approx(float((res["zncc"] >= 0).mean()), abs=1e-6)
        assert entry["bad_ratio"] == pytest.approx(rep["bad_after_repair"] / len(res), abs=1e-6)
        assert (entry["baseline_bad_ratio"] is not None) and entry["fallback_threshold"] == pytest.approx(
            entry["baseline_bad_ratio"] + 0.03, abs=1e-6)
        # against the synthetic truth: the reference's subpixel gate kind of check
        u, v = fields[k](rec["x"].astype(np.float64), rec["y"].astype(np.float64))
        ok = rec["zncc"] >= 0
        assert ok.mean() > 0.95
        assert np.median(np.abs(rec["u"][ok] - u[ok])) < 0.02 and np.median(np.abs(rec["v"][ok] - v[ok])) < 0.02


def test_csv_and_filters(dic, cli, stream12, tmp_path):
    d, ref, tars, _ = stream12
    out = tmp_path / "csv"
    rc, status, err = F.run_cli(cli, ["--multi-frame", "--ref", d / "ref.pgm", "--tar-list", d / "tar_list.txt",
                                      "--output-dir", out, "12", "8", "--input-depth", "12", "--quiet", "--no-preload",
                                      "--output-roi", "40,30,200,150", "--output-step", "2"])
    assert rc == 0, err
    assert not (out / "manifest.opencorr-raw.json").exists() and "[2/6]" not in err
    want = engine_sequence(dic, ref, tars, 12, 8)
    for k, (res, _) in enumerate(want):
        got = F.read_csv(out / f"frame_{k:06d}.csv")
        x, y = res["x"].astype(int), res["y"].astype(int)
        keep = (x >= 40) & (x <= 200) & (y >= 30) & (y <= 150) & (x % 2 == 0) & (y % 2 == 0)
        sel = res[keep]
        assert len(got) == keep.sum() > 0
        np.testing.assert_array_equal(got["x"], sel["x"])
        for name in ("u", "v", "zncc", "ux", "uy", "vx", "vy"):
            # six significant digits, as the reference prints them
            np.testing.assert_allclose(got[name], sel[name], rtol=1e-5, atol=1e-30)


def test_line_mode_and_no_skip(dic, cli, stream12, tmp_path):
    d, ref, tars, _ = stream12
    out = tmp_path / "line"
    lines = [100, 40, 100, 3]       # given order, repeats kept, rows inside the margin only
    rc, _, err = F.run_cli(cli, ["--multi-frame", "--ref", d / "ref.pgm", "--tar-list", d / "tar_list.txt",
                                 "--output-dir", out, "12", "8", "--input-depth", "12", "--line", "100,40",
                                 "--line", "100,3", "--no-skip-fftcc", "--output-format", "raw"])
    assert rc == 0, err
    want = engine_sequence(dic, ref, tars, 12, 8, lines=lines, skip=False)
    frames = list(F.iter_frames(out / "manifest.opencorr-raw.json"))
    assert frames[0][1]["y"].tolist()[:2] == [100, 100]
    for (entry, rec), (res, _) in zip(frames, want):
        assert entry["skip_fftcc_used"] is False and entry["baseline_bad_ratio"] is None
        np.testing.assert_array_equal(rec["u"], res["u"])
        np.testing.assert_array_equal(rec["zncc"], res["zncc"])


def test_single_frame_raw_and_left_aligned_12_bit(dic, cli, tmp_path, oracle_mod):
    from fasticgn_gb300 import speckle
    O = oracle_mod
    pr = speckle.pair_affine(seed=9, width=256, height=256)
    ref16, tar16 = pr.ref.astype(np.uint16) * 16 * 16, pr.tar.astype(np.uint16) * 16 * 16   # 12-bit left-aligned
    F.write_tiff(tmp_path / "ref.tif", ref16)
    F.write_tiff(tmp_path / "tar.tif", tar16, big_endian=True)
    rc, status, err = F.run_cli(cli, [tmp_path / "ref.tif", tmp_path / "tar.tif", "15", "8", tmp_path / "res" / "pair.csv",
                                      "--input-depth", "12", "--output-format", "raw", "--diagnostics"])
    assert rc == 0, err
    assert status["mode"] == "single-frame" and status["output_path"].endswith("pair.bin")
    assert "effective_align=left" in err and "scale=0.0625" in err
    m = F.read_manifest(tmp_path / "res" / "pair.bin.manifest.json")
    entry, rec = next(F.iter_frames(tmp_path / "res" / "pair.bin.manifest.json"))
    # left-aligned 12-bit read with scale 1/16 is the 8-bit pair times 16: same solution as the
    # CPU path on the 12-bit values
    pois = O.grid_pois(256, 256, 15, 8)
    O.run_pair((ref16 / 16.0).astype(np.float32), (tar16 / 16.0).astype(np.float32), pois, 15)
    res = C.compare_frame({"u": pois["p"][:, O.P_U], "v": pois["p"][:, O.P_V], "zncc": pois["r"][:, O.R_ZNCC]},
                          {"u": rec["u"], "v": rec["v"], "zncc": rec["zncc"]})
    assert res["pass"], res
    # diagnostics beside the output: <stem>.diagnostics/<stem>.diagnostics.csv plus its manifest
    ddir = tmp_path / "res" / "pair.diagnostics"
    diag = (ddir / "pair.diagnostics.csv").read_text().splitlines()
    assert diag[0] == "x,y,iteration,convergence,status,zncc" and len(diag) == len(rec) + 1
    dm = json.loads((ddir / "manifest.opencorr-diagnostics.json").read_text())
    assert dm["format"] == "opencorr-gpu-diagnostics-csv-v1" and dm["frames"][0]["file"] == "pair.diagnostics.csv"
    assert dm["frames"][0]["rows"] == len(rec) and dm["columns"][-1] == "zncc"
    assert m["frames"][0]["rows"] == len(rec)


def test_bad_frame_keeps_earlier_frames(dic, cli, stream12, tmp_path):
    """A target that cannot be decoded fails the run (exit 1, status line with the error)
    after the frames before it are written."""
    d, ref, tars, _ = stream12
    bad = tmp_path / "bad.pgm"
    bad.write_bytes(b"P5\n10 10\n255\n" + b"\x00" * 7)     # truncated
    lines = [f"{d / 'tar 000.pgm'} frame_000000.csv", f"{d / 'tar 001.pgm'} frame_000001.csv",
             f"{bad} frame_000002.csv", f"{d / 'tar 003.pgm'} frame_000003.csv"]
    (tmp_path / "list.txt").write_text("\n".join(lines) + "\n")
    out = tmp_path / "out"
    rc, status, err = F.run_cli(cli, ["--multi-frame", "--ref", d / "ref.pgm", "--tar-list", tmp_path / "list.txt",
                                      "--output-dir", out, "12", "8", "--input-depth", "12", "--output-format", "raw"])
    assert rc == 1 and status["status"] == "error" and "truncated PGM" in status["error"], status
    assert status["frames_processed"] == 2
    assert (out / "frame_000000.bin").exists() and (out / "frame_000001.bin").exists()
    assert not (out / "frame_000002.bin").exists() and not (out / "manifest.opencorr-raw.json").exists()
    rc, v, _ = verify(cli, out)
    assert rc == 1 and v["status"] == "incomplete" and v["frames_verified"] == 2 and v["missing_count"] == 2
    assert v["manifests"][0]["state"] == "missing" and v["completion"]["state"] == "missing"


def verify(cli, d):
    p = subprocess.run([str(cli), "--verify-only", str(d)], capture_output=True, text=True)
    return p.returncode, json.loads(p.stdout.strip().splitlines()[-1]), p.stderr


def multi_args(d, out, *extra, tar_list=None):
    return ["--multi-frame", "--ref", d / "ref.pgm", "--tar-list", tar_list or d / "tar_list.txt", "--output-dir", out,
            "12", "8", "--input-depth", "12", "--output-format", "raw", *extra]


def snapshot(out):
    return {p.name: (p.read_bytes(), p.stat().st_ino, p.stat().st_mtime_ns) for p in sorted(out.glob("frame_*.bin"))}


def test_ledger_rerun_resume_and_repair(cli, stream12, tmp_path):
    """The same command again verifies without computing; a deleted frame is replayed bit for
    bit from frame 1; a corrupt one is refused until --repair quarantines and regenerates it."""
    d, _, _, _ = stream12
    out = tmp_path / "out"
    rc, status, err = F.run_cli(cli, multi_args(d, out))
    assert rc == 0, err
    first = snapshot(out)
    rc, v, _ = verify(cli, out)
    assert rc == 0 and v["status"] == "complete" and v["frames_verified"] == 6 and v["manifests"][0]["state"] == "ok"
    assert v["inputs"]["status"] == "match" and v["inputs"]["checked"] == 7
    # rerun: nothing computed or rewritten
    rc, status, err = F.run_cli(cli, multi_args(d, out))
    assert rc == 0 and "Verified complete run" in err, err
    assert status["frames_processed"] == 0 and status["frames_skipped"] == 6
    assert snapshot(out) == first
    # a deleted frame: replay from frame 1, the others keep their inodes
    (out / "frame_000003.bin").unlink()
    rc, status, err = F.run_cli(cli, multi_args(d, out))
    assert rc == 0 and "Resume: 5 verified files" in err, err
    assert status["totals"]["resumed_from_existing_files"] == 5
    assert snapshot(out)["frame_000003.bin"][0] == first["frame_000003.bin"][0]
    assert {k: v[1:] for k, v in snapshot(out).items() if k != "frame_000003.bin"} == \
           {k: v[1:] for k, v in first.items() if k != "frame_000003.bin"}
    # a corrupt frame: refused, then repaired
    b = bytearray((out / "frame_000001.bin").read_bytes())
    b[40] ^= 0x01
    (out / "frame_000001.bin").write_bytes(bytes(b))
    rc, status, err = F.run_cli(cli, multi_args(d, out))
    assert rc == 1 and "corrupt/truncated output" in status["error"] and "--repair" in status["error"]
    rc, v, _ = verify(cli, out)
    assert v["status"] == "damaged" and v["mismatched"] == ["frame_000001.bin"]
    rc, status, err = F.run_cli(cli, multi_args(d, out, "--repair"))
    assert rc == 0 and "Repair: quarantined 1" in err, err
    assert (out / "frame_000001.bin").read_bytes() == first["frame_000001.bin"][0]
    assert verify(cli, out)[1]["status"] == "complete"
    # an option that decides the output bytes
    rc, status, err = F.run_cli(cli, multi_args(d, out, "--max-iter", "11"))
    assert rc == 1 and "options.max_iteration: 10 -> 11" in status["error"], status
    # scheduling options and the durability policy are not part of the contract
    rc, status, err = F.run_cli(cli, multi_args(d, out, "--no-preload", "--durability", "fsync", "--threads", "3"))
    assert rc == 0 and status["frames_skipped"] == 6, err


def test_ledger_append_equals_one_run(cli, stream12, tmp_path):
    """A target list extended by appending continues the run; its frames equal the frames of
    one uninterrupted run over the whole list (the replay restores the temporal state)."""
    d, _, _, _ = stream12
    whole = tmp_path / "whole"
    assert F.run_cli(cli, multi_args(d, whole))[0] == 0
    lines = (d / "tar_list.txt").read_text().splitlines()
    part = tmp_path / "part"
    short = tmp_path / "short.txt"
    short.write_text("\n".join(lines[:4]) + "\n")
    assert F.run_cli(cli, multi_args(d, part, tar_list=short))[0] == 0
    rc, status, err = F.run_cli(cli, multi_args(d, part))
    assert rc == 0 and "Resume: 4 verified files" in err, err
    assert {k: v[0] for k, v in snapshot(part).items()} == {k: v[0] for k, v in snapshot(whole).items()}
    assert verify(cli, part)[1]["status"] == "complete"
    rc, status, _ = F.run_cli(cli, multi_args(d, part, tar_list=short))
    assert rc == 1 and "a shorter list is not a resume" in status["error"]


def test_ledger_diagnostics_csv_run(cli, stream12, tmp_path):
    d, _, _, _ = stream12
    out = tmp_path / "csv"
    args = ["--multi-frame", "--ref", d / "ref.pgm", "--tar-list", d / "tar_list.txt", "--output-dir", out, "12", "8",
            "--input-depth", "12", "--diagnostics", "--quiet"]
    rc, status, err = F.run_cli(cli, args)
    assert rc == 0, err
    files = sorted(p.name for p in (out / "diagnostics").iterdir())
    assert files == sorted([f"frame_{k:06d}.diagnostics.csv" for k in range(6)] + ["manifest.opencorr-diagnostics.json"])
    rc, v, _ = verify(cli, out)
    assert rc == 0 and v["status"] == "complete" and v["files_expected"] == 13   # 6 CSV, 6 diagnostics, 1 manifest
    assert F.run_cli(cli, args)[2].count("Verified complete run") == 1


def test_temporal_extrapolation_run(dic, cli, tmp_path):
    """--temporal-extrapolation: records equal the engine's temporal sequence; the manifest's
    per-frame QA and the status totals count the extrapolated seeds."""
    from fasticgn_gb300 import speckle
    d = tmp_path / "in"
    d.mkdir()
    ref, frames = speckle.stream_frames(width=256, height=224, frames=4, which=[0, 1, 2, 3, 4])
    F.write_pgm(d / "ref.pgm", ref, maxval=4095)
    lines = []
    for k, tar, _ in frames:
        F.write_pgm(d / f"t{k}.pgm", tar, maxval=4095)
        lines.append(f"{d / f't{k}.pgm'} frame_{k:06d}.csv")
    (d / "list.txt").write_text("\n".join(lines) + "\n")
    out = tmp_path / "out"
    rc, status, err = F.run_cli(cli, ["--multi-frame", "--ref", d / "ref.pgm", "--tar-list", d / "list.txt",
                                      "--output-dir", out, "12", "8", "--input-depth", "12", "--output-format", "raw",
                                      "--temporal-extrapolation"])
    assert rc == 0, err
    m = F.read_manifest(out / "manifest.opencorr-raw.json")
    assert m["engine"]["temporal_extrapolation"] is True
    counts = [f["temporal_seed_count"] for f in m["frames"]]
    assert counts[:2] == [0, 0] and all(c > 0 for c in counts[2:]), counts
    assert [f["temporal_seed_used"] for f in m["frames"]] == [c > 0 for c in counts]
    assert status["totals"]["temporal_seed_frames"] == 3 and status["totals"]["temporal_seed_pois"] == sum(counts)
    tmpl = dic.grid_queue(256, 224, 12, 8)
    e = dic.Engine(12)
    e.set_ref(ref)
    e.sequence_begin(tmpl, temporal_extrapolation=True)
    for (entry, rec), (_, tar, _) in zip(F.iter_frames(out / "manifest.opencorr-raw.json"), frames):
        res = np.zeros_like(tmpl)
        rep = e.sequence_frame(tar, res)
        np.testing.assert_array_equal(rec["u"], res["u"])
        np.testing.assert_array_equal(rec["zncc"], res["zncc"])
        assert entry["temporal_seed_count"] == rep["temporal_seed_count"]
    e.close()
    c = json.loads((out / ".opencorr-state" / "contract.json").read_text())
    assert c["options"]["temporal_extrapolation"] is True


@pytest.mark.parametrize("extra", [["--decode-threads", "3"], ["--decode-threads", "2", "--no-preload"]])
def test_decode_threads_do_not_change_outputs(cli, stream12, tmp_path, extra):
    """--decode-threads only schedules the decode (frames are handed out in list order), so
    every payload byte equals the one-worker run's."""
    d, _, _, _ = stream12
    outs = []
    for name, flags in (("one", []), ("many", extra)):
        out = tmp_path / name
        rc, status, err = F.run_cli(cli, ["--multi-frame", "--ref", d / "ref.pgm", "--tar-list", d / "tar_list.txt",
                                          "--output-dir", out, "12", "8", "--input-depth", "12", "--output-format",
                                          "raw", "--quiet", *flags])
        assert rc == 0 and status["frames_processed"] == 6, err
        outs.append(out)
    files = [[f["file"] for f in F.read_manifest(o / "manifest.opencorr-raw.json")["frames"]] for o in outs]
    assert len(files[0]) == 6 and files[0] == files[1]
    for n in files[0]:
        assert (outs[0] / n).read_bytes() == (outs[1] / n).read_bytes(), n

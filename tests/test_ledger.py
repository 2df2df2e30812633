"""The output ledger on the CPU (no GPU): its XXH3-128 against golden digests of the
reference's vendored xxHash, and its run semantics (docs/output-integrity.md of the
reference) through tests/ledger_main.cpp, a synthetic multi-frame run that publishes
through the same RunLedger / audit code as the command line: verified rerun, replay of a
missing frame, --repair of a corrupt one, contract and target-list rejections, appends,
foreign entries, crash residue, locks, changed inputs and manifests."""
import fcntl
import json
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CLI = ROOT / "fasticgn_gb300" / "cli"
N, ROWS = 5, 40


def _compile(tmp_path_factory, main, name, extra):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("bin") / name
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", str(CLI), str(ROOT / "tests" / main),
                    *[str(CLI / f) for f in extra], "-o", str(out)], check=True)
    return out


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return _compile(tmp_path_factory, "ledger_main.cpp", "ledger_main", ["ledger.cpp", "json.cpp", "xxh3.cpp"])


def test_xxh3_matches_reference_vectors(tmp_path_factory):
    exe = _compile(tmp_path_factory, "xxh3_main.cpp", "xxh3_main", ["xxh3.cpp"])
    want = dict(line.split() for line in (ROOT / "tests" / "golden" / "xxh3_vectors.txt").read_text().splitlines())
    out = subprocess.run([str(exe), *want.keys()], check=True, capture_output=True, text=True).stdout
    got = dict(line.split() for line in out.splitlines())    # also checks the incremental form (chunks)
    assert got == want


class Run:
    def __init__(self, harness, root):
        self.h, self.root = harness, root
        self.root.mkdir(exist_ok=True)
        self.list = root / "tar_list.txt"
        self.list.write_text("list\n")

    def run(self, frames=N, *args):
        p = subprocess.run([str(self.h), "run", str(self.root), str(self.list), str(frames), str(ROWS), *map(str, args)],
                           capture_output=True, text=True)
        return p.returncode, json.loads(p.stdout.strip().splitlines()[-1]), p.stderr

    def verify(self):
        p = subprocess.run([str(self.h), "verify", str(self.root)], capture_output=True, text=True)
        return json.loads(p.stdout)

    def frame(self, k):
        return self.root / f"frame_{k:06d}.bin"


@pytest.fixture
def done(harness, tmp_path):
    r = Run(harness, tmp_path / "out")
    rc, out, err = r.run()
    assert rc == 0 and out["published"] == N and not out["complete_at_start"], (out, err)
    return r


def test_fresh_run_and_verified_rerun(done):
    v = done.verify()
    assert v["status"] == "complete" and v["frames_verified"] == N and v["files_expected"] == N + 1
    assert v["rows_per_frame"] == ROWS and v["completion"]["state"] == "current"
    assert v["completion"]["durability"] == "rename" and v["untracked"] == ["tar_list.txt"]
    state = done.root / ".opencorr-state"
    assert json.loads((state / "contract.json").read_text())["targets"][0]["file"] == "frame_000000.bin"
    intents = [json.loads(p.read_text()) for p in state.glob("*.json") if len(p.stem) == 32]
    assert sorted(i["key"] for i in intents) == [f"frame/frame_{k:06d}.bin" for k in range(N)]
    assert all(i["bytes"] == ROWS * 36 and i["algorithm"] == "xxh3-128" for i in intents)
    before = [(p.stat().st_ino, p.stat().st_mtime_ns) for p in map(done.frame, range(N))]
    rc, out, _ = done.run()
    assert rc == 0 and out["complete_at_start"] and out["published"] == 0
    assert out["verified_bytes"] > N * ROWS * 36
    assert [(p.stat().st_ino, p.stat().st_mtime_ns) for p in map(done.frame, range(N))] == before


def test_missing_frame_is_replayed(done):
    want = done.frame(2).read_bytes()
    others = [done.frame(k).stat().st_ino for k in (0, 1, 3, 4)]
    done.frame(2).unlink()
    v = done.verify()
    assert v["status"] == "incomplete" and v["missing"] == ["frame_000002.bin"] and v["missing_count"] == 1
    rc, out, _ = done.run()
    assert rc == 0 and out["existing"] == N - 1 and out["published"] == 1
    assert done.frame(2).read_bytes() == want
    assert [done.frame(k).stat().st_ino for k in (0, 1, 3, 4)] == others
    assert done.verify()["status"] == "complete"


def test_corrupt_frame_needs_repair(done):
    want = done.frame(1).read_bytes()
    bad = bytearray(want)
    bad[100] ^= 0x40                                     # same size, different content
    done.frame(1).write_bytes(bytes(bad))
    rc, out, _ = done.run()
    assert rc == 1 and "corrupt/truncated output; resume refused" in out["error"] and "--repair" in out["error"]
    v = done.verify()
    assert v["status"] == "damaged" and v["mismatched"] == ["frame_000001.bin"]
    assert done.frame(1).read_bytes() == bytes(bad)      # a rejected run changes nothing
    rc, out, _ = done.run(N, "--repair")
    assert rc == 0 and out["quarantined"] == 1 and out["published"] == 1
    assert done.frame(1).read_bytes() == want
    moved = list(Path(out["quarantine_dir"]).iterdir())
    assert [p.name for p in moved] == ["frame_000001.bin"] and moved[0].read_bytes() == bytes(bad)
    assert done.verify()["status"] == "complete"


def test_truncated_frame_and_no_intent(done):
    done.frame(3).write_bytes(done.frame(3).read_bytes()[:-7])
    assert "corrupt/truncated output" in done.run()[1]["error"]
    intent = [p for p in (done.root / ".opencorr-state").glob("*.json")
              if len(p.stem) == 32 and json.loads(p.read_text())["key"] == "frame/frame_000004.bin"][0]
    intent.unlink()
    v = done.verify()
    assert v["status"] == "damaged" and v["mismatched"] == ["frame_000003.bin"] and v["no_intent"] == ["frame_000004.bin"]
    rc, out, _ = done.run(N, "--repair")
    assert rc == 0 and out["quarantined"] == 2
    assert done.verify()["status"] == "complete"


def test_changed_option_is_rejected(done):
    rc, out, _ = done.run(N, "--option", "2")
    assert rc == 1
    assert out["error"].startswith("resume rejected: run configuration/reference/binary changed (recorded -> requested): "
                                   'options.option: "1" -> "2"')
    assert "an option that decides the output differs" in out["error"]
    assert done.verify()["status"] == "complete"         # nothing changed


def test_target_list_shorter_rejected_longer_appends(done):
    rc, out, _ = done.run(N - 1)
    assert rc == 1 and "a shorter list is not a resume" in out["error"]
    rc, out, _ = done.run(N + 2)
    assert rc == 0 and out["existing"] == N and out["published"] == 2
    v = done.verify()
    assert v["status"] == "complete" and v["frames_verified"] == N + 2
    assert not (done.root / ".opencorr-state" / "contract.pending.json").exists()


def test_interrupted_appends(done):
    # stopped before any new output: the pending contract waits, the old run is still complete
    rc, out, _ = done.run(N + 2, "--stop-after", N)
    assert rc == 0 and out["stopped"]
    assert (done.root / ".opencorr-state" / "contract.pending.json").exists()
    v = done.verify()
    assert v["status"] == "complete" and v["pending_append"] and v["pending_append_state"] == "append"
    assert any("append was started and stopped" in w for w in v["warnings"])
    # stopped after the first new output: the longer contract was promoted with it
    rc, out, _ = done.run(N + 3, "--stop-after", N + 1)
    assert rc == 0 and out["published"] == 1
    v = done.verify()
    assert v["status"] == "incomplete" and v["completion"]["state"] == "other_contract" and v["missing_count"] == 2
    rc, out, _ = done.run(N)                              # the shorter list no longer accounts for the new frame
    assert rc == 1 and "a shorter list is not a resume" in out["error"]
    rc, out, _ = done.run(N + 3)
    assert rc == 0 and out["existing"] == N + 1 and out["published"] == 2
    assert done.verify()["status"] == "complete"


def test_foreign_entries(done):
    (done.root / "notes.txt").write_text("x")
    v = done.verify()
    assert v["status"] == "complete" and "notes.txt" in v["untracked"]
    rc, out, _ = done.run()
    assert rc == 1 and "untracked entry in output directory" in out["error"]
    (done.root / "notes.txt").unlink()
    (done.root / "frame_999999.bin").write_bytes(b"\0" * 36)
    v = done.verify()
    assert v["status"] == "damaged" and v["untracked_outputs"] == ["frame_999999.bin"]


def test_residue_is_archived(done):
    tmp = done.root / ".opencorr-tmp-123-4"
    tmp.write_bytes(b"partial")
    odd = done.root / ".opencorr-tmp-x"
    odd.write_bytes(b"?")
    v = done.verify()
    assert v["status"] == "complete" and sorted(v["residue"]) == [".opencorr-tmp-123-4", ".opencorr-tmp-x"]
    rc, out, err = done.run()
    assert rc == 0 and out["complete_at_start"] and not tmp.exists() and odd.exists()
    assert "leaving unrecognized reserved name in place" in err and "Archived 1 abandoned private file" in err
    assert (Path(out["quarantine_dir"]) / ".opencorr-tmp-123-4").read_bytes() == b"partial"


def test_lock_excludes_runs_and_audits(done):
    fd = os.open(done.root, os.O_RDONLY | os.O_DIRECTORY)
    try:
        fcntl.flock(fd, fcntl.LOCK_EX | fcntl.LOCK_NB)
        rc, out, _ = done.run()
        assert rc == 1 and "run directory already locked" in out["error"]
        assert done.verify()["status"] == "locked"
    finally:
        os.close(fd)
    assert done.verify()["status"] == "complete"


def test_stray_output_without_record(harness, tmp_path):
    r = Run(harness, tmp_path / "fresh")
    r.frame(0).write_bytes(b"\0" * 36 * ROWS)
    rc, out, _ = r.run()
    assert rc == 1 and "existing output has no verified run record" in out["error"]
    assert r.verify()["status"] == "not_a_run"


def test_changed_input_and_manifest(harness, tmp_path):
    r = Run(harness, tmp_path / "inp")
    img = tmp_path / "ref.pgm"
    img.write_bytes(b"P5\n2 2\n255\n\0\1\2\3")
    assert r.run(N, "--input", img)[0] == 0
    img.write_bytes(b"P5\n2 2\n255\n\0\1\2\4")
    v = r.verify()
    assert v["status"] == "inputs_changed" and v["inputs"]["changed"] == [str(img.resolve())]
    rc, out, _ = r.run(N, "--input", img)
    assert rc == 1 and "the reference image path or content differs" in out["error"]
    r2 = Run(harness, tmp_path / "man")
    assert r2.run()[0] == 0
    m = r2.root / "manifest.opencorr-raw.json"
    doc = json.loads(m.read_text())
    doc["frames"][0]["rows"] = 1
    m.write_text(json.dumps(doc))
    v = r2.verify()
    assert v["status"] == "damaged" and v["manifests"][0]["state"] == "changed"
    rc, out, _ = r2.run()
    assert rc == 1 and "completed manifest changed" in out["error"]
    rc, out, _ = r2.run(N, "--repair")
    assert rc == 0 and out["quarantined"] == 2            # the completion record and that manifest
    assert r2.verify()["status"] == "complete"
    # whitespace-only reformatting of a manifest is not a change
    m.write_text(json.dumps(json.loads(m.read_text()), indent=4))
    assert r2.verify()["status"] == "complete"


def test_replay_must_reproduce_recorded_bytes(done):
    done.frame(4).unlink()
    rc, out, _ = done.run(N, "--corrupt-replay", 2)
    assert rc == 1 and "replayed bytes differ from recorded output" in out["error"]


def test_fsync_policy_and_durability_record(harness, tmp_path):
    r = Run(harness, tmp_path / "fs")
    assert r.run(N, "--fsync")[0] == 0
    assert r.verify()["completion"]["durability"] == "fsync"
    rc, out, _ = r.run(N)                                # the policy is not part of the contract
    assert rc == 0 and out["complete_at_start"]

"""GPU tests of the frame policy (processFrame, opencorr_cli_cuda_mvp.cpp:3024-3210) and of
fixed-reference sequences, against the oracle restatement in oracle/frame_policy.py."""
import numpy as np
import pytest

import dic_checks as C

pytestmark = pytest.mark.gpu


def to_oracle(O, q):
    pois = np.zeros(len(q), dtype=O.POI2D_DTYPE)
    pois["x"], pois["y"] = q["x"], q["y"]
    for name, idx in (("u", O.P_U), ("ux", O.P_UX), ("uy", O.P_UY), ("v", O.P_V), ("vx", O.P_VX), ("vy", O.P_VY)):
        pois["p"][:, idx] = q[name]
    for name, idx in (("u0", O.R_U0), ("v0", O.R_V0), ("zncc", O.R_ZNCC), ("iteration", O.R_ITER),
                      ("convergence", O.R_CONV)):
        pois["r"][:, idx] = q[name]
    return pois


def oracle_fields(O, pois):
    return {"u": pois["p"][:, O.P_U], "v": pois["p"][:, O.P_V], "zncc": pois["r"][:, O.R_ZNCC]}


def shifted(img, dx, dy, fill=127):
    """generate_synthetic_dic.shifted_image: dst(x, y) = src(x - dx, y - dy), fill outside."""
    out = np.full_like(img, fill)
    h, w = img.shape
    out[max(0, dy):min(h, h + dy), max(0, dx):min(w, w + dx)] = \
        img[max(0, -dy):min(h, h - dy), max(0, -dx):min(w, w - dx)]
    return out


def test_sequence_matches_policy_oracle(dic, oracle_mod):
    """A 12-bit stream: frame 0 by FFTCC + IC-GN, later frames seeded from the previous one."""
    O = oracle_mod
    from oracle import frame_policy as FP
    from fasticgn_gb300 import speckle
    ref, frames = speckle.stream_frames(width=256, height=256, frames=200, which=[0, 1, 2, 3, 4, 5])
    tars = [f[1] for f in frames]
    radius, step = 12, 8
    tmpl = dic.grid_queue(256, 256, radius, step)
    e = dic.Engine(radius)
    e.set_ref(ref)
    e.sequence_begin(tmpl)
    got = []
    for tar in tars:
        res = np.zeros_like(tmpl)
        rep = e.sequence_frame(tar, res)
        got.append((res, rep))
    want = FP.run_sequence(ref, tars, to_oracle(O, tmpl), radius)
    for k, ((g, rep), (w, info)) in enumerate(zip(got, want)):
        r = C.compare_frame(oracle_fields(O, w), {"u": g["u"], "v": g["v"], "zncc": g["zncc"]})
        assert r["pass"], (k, r)
        assert rep["frame_fallback_used"] == int(info["frame_fallback"]), (k, rep, info)
        assert abs(rep["bad_before_repair"] - info["bad"]) <= 2, (k, rep, info)
    # only the first frame runs FFTCC; the seeded frames converge without it
    assert got[0][1]["fftcc_used"] == 1 and all(rep["fftcc_used"] == 0 for _, rep in got[1:])


def test_sequence_graph_equals_eager(dic):
    from fasticgn_gb300 import speckle
    ref, frames = speckle.stream_frames(width=192, height=192, frames=4, which=[0, 1, 2, 3])
    tmpl = dic.grid_queue(192, 192, 10, 6)
    outs = []
    for graphs in (True, False):
        e = dic.Engine(10)
        e.set_graphs(graphs)
        e.set_ref(ref)
        e.sequence_begin(tmpl)
        seq = []
        for _, tar, _ in frames:
            res = np.zeros_like(tmpl)
            e.sequence_frame(tar, res)
            seq.append(res.tobytes())
        outs.append(seq)
    assert outs[0] == outs[1]


def test_jump_triggers_frame_fallback(dic, oracle_mod, golden):
    """A 12 px jump between frames: the seeded attempt fails across the frame, the bad ratio
    exceeds baseline + 0.03, the whole-frame FFTCC + IC-GN pass runs and the merge never
    raises the bad count."""
    O = oracle_mod
    from oracle import frame_policy as FP
    g = golden("oob")
    ref = g["ref"]
    h, w = ref.shape
    tars = [ref, shifted(ref, 12, 0)]
    radius = 15
    tmpl = dic.grid_queue(w, h, radius, 4)
    e = dic.Engine(radius)
    e.set_ref(ref)
    e.sequence_begin(tmpl)
    reps, outs = [], []
    for tar in tars:
        res = np.zeros_like(tmpl)
        reps.append(e.sequence_frame(tar, res))
        outs.append(res)
    assert reps[1]["frame_fallback_used"] == 1
    assert reps[1]["bad_after_repair"] <= reps[1]["bad_before_repair"]
    want = FP.run_sequence(ref, tars, to_oracle(O, tmpl), radius)
    assert want[1][1]["frame_fallback"]
    r = C.compare_frame(oracle_fields(O, want[1][0]), {"u": outs[1]["u"], "v": outs[1]["v"], "zncc": outs[1]["zncc"]},
                        min_shared_valid=50)
    assert r["pass"], r
    ok = outs[1]["zncc"] >= 0.8
    assert np.median(np.abs(outs[1]["u"][ok] - 12.0)) < 1e-3


def test_poi_level_repair(dic, oracle_mod, affine_pair_small):
    """A few previous results off by 6 px: IC-GN from those seeds goes bad, the POIs are
    repair candidates (previous zncc >= 0.8), and FFTCC + IC-GN on just those recovers them."""
    O = oracle_mod
    from oracle import frame_policy as FP
    pr = affine_pair_small
    h, w = pr.ref.shape
    radius = 15
    tmpl = dic.grid_queue(w, h, radius, 10)
    e = dic.Engine(radius)
    e.set_ref(pr.ref)
    e.set_tar(pr.tar)
    prev = tmpl.copy()
    e.process_pair(prev)
    bad_idx = np.arange(40, len(prev), 97)[:12]
    prev["u"][bad_idx] += 6.0
    q = tmpl.copy()
    q, rep = e.process_frame(q, prev, skip_fftcc=True, poi_fallback=True, frame_fallback_ratio=0.5)
    assert rep["frame_fallback_used"] == 0
    # POIs pushed out of range by the wrong seed end -3, which is not "bad" (-3 is terminal
    # at POI level); the others are candidates
    assert rep["repaired_candidates"] >= 1
    assert rep["bad_after_repair"] < rep["bad_before_repair"]
    solver = FP.Solver(pr.ref, radius)
    solver.set_tar(pr.tar)
    oq, info = FP.process_frame(solver, to_oracle(O, tmpl), to_oracle(O, prev), True, True, 0.5)
    assert info["candidates"] == rep["repaired_candidates"]
    r = C.compare_frame(oracle_fields(O, oq), {"u": q["u"], "v": q["v"], "zncc": q["zncc"]}, min_shared_valid=50)
    assert r["pass"], r
    z = q["zncc"][bad_idx]
    assert np.all((z == -3.0) | (z >= 0.8))


@pytest.fixture(scope="module")
def affine_pair_small():
    from fasticgn_gb300 import speckle
    return speckle.pair_affine(seed=3, width=384, height=320)


def temporal_stream():
    from fasticgn_gb300 import speckle
    # 4 frames to full amplitude: the displacement grows ~0.125 px per frame, so most POIs
    # take the extrapolated seed from frame 2 on
    ref, frames = speckle.stream_frames(width=256, height=256, frames=4, which=[0, 1, 2, 3, 4, 5])
    return ref, [f[1] for f in frames]


def test_temporal_sequence_matches_policy_oracle(dic, oracle_mod):
    """Skip-FFTCC frames seeded by temporal extrapolation from the two previous results
    (seedPoiQueueFromPrevious, :594-616), against the restated policy frame by frame."""
    O = oracle_mod
    from oracle import frame_policy as FP
    ref, tars = temporal_stream()
    radius, step = 12, 8
    tmpl = dic.grid_queue(256, 256, radius, step)
    e = dic.Engine(radius)
    e.set_ref(ref)
    e.sequence_begin(tmpl, temporal_extrapolation=True)
    got = []
    for tar in tars:
        res = np.zeros_like(tmpl)
        rep = e.sequence_frame(tar, res)
        got.append((res, rep))
    e.close()
    want = FP.run_sequence(ref, tars, to_oracle(O, tmpl), radius, temporal=True)
    for k, ((g, rep), (w, info)) in enumerate(zip(got, want)):
        r = C.compare_frame(oracle_fields(O, w), {"u": g["u"], "v": g["v"], "zncc": g["zncc"]})
        assert r["pass"], (k, r)
        # the counts depend on results equal to ~1e-6 px: equal up to a POI or two at the thresholds
        assert abs(rep["temporal_seed_count"] - info["temporal"]) <= 2, (k, rep, info)
    counts = [rep["temporal_seed_count"] for _, rep in got]
    assert counts[0] == 0 and counts[1] == 0 and min(counts[2:]) > 0.3 * len(tmpl), counts


def test_temporal_graph_equals_eager_and_off_differs(dic):
    ref, tars = temporal_stream()
    tmpl = dic.grid_queue(256, 256, 12, 8)
    outs = {}
    for graphs, temporal in ((True, True), (False, True), (True, False)):
        e = dic.Engine(12)
        e.set_graphs(graphs)
        e.set_ref(ref)
        e.sequence_begin(tmpl, temporal_extrapolation=temporal)
        seq = []
        for tar in tars:
            res = np.zeros_like(tmpl)
            e.sequence_frame(tar, res)
            seq.append(res.copy())
        e.close()
        outs[(graphs, temporal)] = seq
    for a, b in zip(outs[(True, True)], outs[(False, True)]):
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))
    # the seed changes where IC-GN starts: frames 0-1 equal, later frames not bit-identical
    for k in (0, 1):
        np.testing.assert_array_equal(outs[(True, True)][k].view(np.uint8), outs[(True, False)][k].view(np.uint8))
    assert not np.array_equal(outs[(True, True)][3].view(np.uint8), outs[(True, False)][3].view(np.uint8))


def test_process_frame_history_matches_oracle(dic, oracle_mod):
    O = oracle_mod
    from oracle import frame_policy as FP
    ref, tars = temporal_stream()
    radius, step = 12, 8
    tmpl = dic.grid_queue(256, 256, radius, step)
    e = dic.Engine(radius)
    e.set_ref(ref)
    hist = []
    for tar in tars[:2]:
        e.set_tar(tar)
        q = tmpl.copy()
        e.process_pair(q)
        hist.append(q)
    e.set_tar(tars[2])
    q, rep = e.process_frame(tmpl.copy(), hist[1], prev_prev=hist[0], temporal_extrapolation=True)
    e.close()
    solver = FP.Solver(ref, radius)
    solver.set_tar(tars[2])
    oq, info = FP.process_frame(solver, to_oracle(O, tmpl), to_oracle(O, hist[1]), True, True,
                                prev2=to_oracle(O, hist[0]), temporal=True)
    assert rep["temporal_seed_count"] > 0 and abs(rep["temporal_seed_count"] - info["temporal"]) <= 2
    r = C.compare_frame(oracle_fields(O, oq), {"u": q["u"], "v": q["v"], "zncc": q["zncc"]})
    assert r["pass"], r

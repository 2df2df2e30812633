"""Parity at the streams' own sizes, against the CPU oracle.

* 2048x2048 12-bit sine/strain stream, subset radius 15, POI step 5 (162 409 POIs per frame):
  four consecutive frames of the 200-frame ramp through the sequence API (the first by
  FFTCC + IC-GN, the others seeded from the previous frame with POI repair and the
  whole-frame fallback), against the restated processFrame loop (oracle/frame_policy.py,
  opencorr_cli_cuda_mvp.cpp:3024-3210) over the whole queue.
* 1024x1024 12-bit crack stream, subset radius 12, POI step 4 (62 001 POIs per frame): three
  consecutive frames through learned-seed sequences (proposal seeds, IC-GN capped at 6
  iterations, FFTCC + IC-GN below ZNCC 0.9), each against the oracle's FFTCC + IC-GN on the
  same frame over the whole queue; the converged IC-GN is the judge of the proposal.

Each frame must pass the reference parity gate (smoke/check_cpu_gpu_parity.py:46-98: median
|du|,|dv| <= 1e-3 px, p99 <= 1e-2 px, max <= 0.5 px, retention >= 0.95, validity
disagreement <= 0.05), and the failure flags must agree.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

import dic_checks as C

pytestmark = pytest.mark.gpu


def render(kind, seed, width, height, frames, which):
    """Reference + frames of a stream, rendered by a spawn pool (no fork after CUDA use)."""
    from fasticgn_gb300 import speckle
    specs = [(kind, seed, width, height, frames, k) for k in [-1] + list(which)]
    with mp.get_context("spawn").Pool(min(len(specs), os.cpu_count() or 1)) as pool:
        imgs = pool.map(speckle.stream_image, specs, chunksize=1)
    return imgs[0], imgs[1:]


def to_oracle(O, q):
    pois = np.zeros(len(q), dtype=O.POI2D_DTYPE)
    pois["x"], pois["y"] = q["x"], q["y"]
    for name, idx in (("u", O.P_U), ("ux", O.P_UX), ("uy", O.P_UY), ("v", O.P_V), ("vx", O.P_VX), ("vy", O.P_VY)):
        pois["p"][:, idx] = q[name]
    return pois


def oracle_fields(O, pois):
    return {"u": pois["p"][:, O.P_U], "v": pois["p"][:, O.P_V], "zncc": pois["r"][:, O.R_ZNCC],
            "u0": pois["r"][:, O.R_U0], "v0": pois["r"][:, O.R_V0]}


@pytest.fixture(scope="module")
def stream2048():
    # frames 100..103 of 200: the middle of the bench window
    return render("stream", 2, 2048, 2048, 200, [100, 101, 102, 103])


@pytest.fixture(scope="module")
def crack1024():
    # the last frames of the 5000-frame ramp (crack jump 1.5 px)
    return render("crack", 5, 1024, 1024, 5000, [4997, 4998, 4999])


def test_stream2048_12bit_sequence_matches_policy_oracle(dic, oracle_mod, stream2048):
    O = oracle_mod
    from oracle import frame_policy as FP
    ref, tars = stream2048
    radius, step = 15, 5
    tmpl = dic.grid_queue(2048, 2048, radius, step)
    assert len(tmpl) == 162409
    e = dic.Engine(radius)
    e.set_ref(ref)
    e.sequence_begin(tmpl)
    got = []
    for tar in tars:
        res = np.zeros_like(tmpl)
        rep = e.sequence_frame(tar, res)
        got.append((res, rep))
    e.close()
    want = FP.run_sequence(ref, tars, to_oracle(O, tmpl), radius)
    for k, ((g, rep), (w, info)) in enumerate(zip(got, want)):
        cpu = oracle_fields(O, w)
        r = C.compare_frame(cpu, {"u": g["u"], "v": g["v"], "zncc": g["zncc"]})
        assert r["pass"], (k, r)
        same = np.mean(C.failure_codes(cpu["zncc"]) == C.failure_codes(g["zncc"]))
        assert same >= 0.999, (k, same)
        assert rep["frame_fallback_used"] == int(info["frame_fallback"]), (k, rep, info)
        assert abs(rep["bad_before_repair"] - info["bad"]) <= max(2, len(tmpl) // 20000), (k, rep, info)
        if k == 0:
            C.assert_flags_agree(cpu, {"u0": g["u0"], "v0": g["v0"], "zncc": g["zncc"]})
    # FFTCC runs on the first frame and, later, only for POI repair or a whole-frame fallback
    assert got[0][1]["fftcc_used"] == 1
    for k, (_, rep) in enumerate(got[1:], 1):
        repaired = rep["repaired_candidates"] > 0 or rep["frame_fallback_used"]
        assert rep["fftcc_used"] == int(repaired), (k, rep)


def proposal_seeds(dic, net, ref, tar, tmpl):
    """The network's seeds for one frame (the fused kernel the engine runs), as (n, 6) float32
    columns u, ux, uy, v, vx, vy."""
    import torch
    rf = torch.from_numpy(ref.astype(np.float32)).cuda()
    tf = torch.from_numpy(tar.astype(np.float32)).cuda()
    qd = torch.from_numpy(tmpl.view(np.uint8).copy()).cuda()
    net.seed(rf, tf, qd, len(tmpl))
    s = qd.cpu().numpy().view(dic.POI_DTYPE)
    return np.stack([s[k] for k in ("u", "ux", "uy", "v", "vx", "vy")], axis=1).astype(np.float32)


def test_crack1024_learned_sequence_matches_oracle(dic, oracle_mod, crack1024):
    """Displacements against the CPU path (FFTCC + IC-GN, the judge of the proposal); failure
    flags against the oracle's run of the same learned-seed policy from the same proposal
    seeds (oracle/frame_policy.learned_policy): a POI's outcome depends on where IC-GN
    starts, so flags are compared from identical starting points."""
    O = oracle_mod
    pytest.importorskip("torch")
    from fasticgn_gb300 import proposal, speckle
    from oracle import frame_policy as FP
    if not proposal.WEIGHTS.exists():
        pytest.skip("no trained weights")
    ref, tars = crack1024
    radius, step = 12, 4
    tmpl = dic.grid_queue(1024, 1024, radius, step)
    assert len(tmpl) == 62001
    net = proposal.ProposalNet.load()
    e = dic.Engine(radius)
    e.set_proposal(net)
    e.set_ref(ref)
    e.sequence_begin(tmpl, learned_seed=True)
    got = []
    for tar in tars:
        res = np.zeros_like(tmpl)
        rep = e.sequence_frame(tar, res)
        got.append((res, rep))
    e.close()
    seeds = [proposal_seeds(dic, net, ref, tar, tmpl) for tar in tars]
    net.close()
    solver = FP.Solver(ref, radius)
    for k, (tar, (g, rep)) in enumerate(zip(tars, got)):
        solver.set_tar(tar)
        pois = to_oracle(O, tmpl)
        solver.fftcc(pois)
        solver.icgn(pois)
        cpu = oracle_fields(O, pois)
        r = C.compare_frame(cpu, {"u": g["u"], "v": g["v"], "zncc": g["zncc"]})
        assert r["pass"], (k, r)
        same, fallbacks = FP.learned_policy(solver, to_oracle(O, tmpl), seeds[k])
        fc, fg = C.failure_codes(same["r"][:, O.R_ZNCC]), C.failure_codes(g["zncc"])
        agree = fc == fg
        detail = [(float(fc[i]), float(fg[i]), float(same["r"][i, O.R_ITER]), float(g["iteration"][i]))
                  for i in np.flatnonzero(~agree)[:10]]
        assert agree.mean() >= 0.999, (k, agree.mean(), detail)
        # the fallback set is the same policy's: POIs below ZNCC 0.9 after the capped IC-GN
        assert abs(rep["repaired_candidates"] - fallbacks) <= max(5, 0.002 * len(tmpl)), (rep, fallbacks)
        assert rep["repaired_candidates"] < 0.2 * len(tmpl), rep

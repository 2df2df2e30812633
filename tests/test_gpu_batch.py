"""GPU tests of the uneven batch (dic_batch_process): pairs of different sizes, pixel types
and subset radii, with very different POI counts, solved through one persistent IC-GN
launch per code path.  Each job is checked against the CPU oracle of the pair (FFTCC seed +
IC-GN, the reference's per-pair path), and bit for bit against the engine's own
single-pair path, which runs the same kernels one pair at a time."""
import numpy as np
import pytest

import dic_checks as C

pytestmark = pytest.mark.gpu


def _jobs():
    """Jobs of the uneven batch's kind at test sizes: per-pair affine fields with 20 % flat
    patches (u8) -- radii 10 and 15 (column walk), 20 and 30 (pair walk), 32 (flat walk) --
    plus a 12-bit u16 pair and a float32 pair with smooth bump fields."""
    from fasticgn_gb300 import speckle
    rng = np.random.default_rng(71)
    out = []
    for w, h, r, n in [(384, 320, 10, 4000), (640, 512, 15, 16000), (300, 420, 20, 1500), (320, 320, 30, 600),
                       (300, 280, 32, 300)]:
        p = speckle.pair_uneven(rng, w, h, r, n)
        out.append((p.ref, p.tar, r, p.step))
    pr = speckle.pair_bumps(seed=73, width=300, height=260, max_disp=6.0, max_strain=0.01)
    out.append((pr.ref.astype(np.uint16) * 16, pr.tar.astype(np.uint16) * 16, 12, 7))
    pr = speckle.pair_bumps(seed=74, width=256, height=288, max_disp=6.0, max_strain=0.01)
    out.append((pr.ref.astype(np.float32), pr.tar.astype(np.float32), 7, 3))
    pr = speckle.pair_bumps(seed=76, width=200, height=180, max_disp=6.0, max_strain=0.01)
    out.append((pr.ref, pr.tar, 15, 50))
    return out


def test_batch_matches_oracle_and_single_pair(dic, oracle_mod):
    O = oracle_mod
    jobs = _jobs()
    queues = [dic.grid_queue(ref.shape[1], ref.shape[0], r, step) for ref, tar, r, step in jobs]
    queues.append(dic.make_queue([], []))   # an empty job
    jobs.append(jobs[0][:2] + (12, 5))
    e = dic.Engine(15)
    batch_q = [q.copy() for q in queues]
    rep = e.batch_process([(ref, tar, r, q) for (ref, tar, r, _), q in zip(jobs, batch_q)])
    assert rep["jobs"] == len(jobs) and rep["pois"] == sum(len(q) for q in queues)
    assert rep["valid"] == sum(int((q["zncc"] >= 0).sum()) for q in batch_q)
    for (ref, tar, r, step), q, got in zip(jobs, queues, batch_q):
        if len(q) == 0:
            continue
        single = q.copy()
        with dic.Engine(r) as s:
            s.set_ref(ref)
            s.set_tar(tar)
            s.process_pair(single)
        for f in ("u", "ux", "uy", "v", "vx", "vy", "zncc", "iteration", "convergence", "u0", "v0"):
            np.testing.assert_array_equal(got[f], single[f], err_msg=f"radius {r} field {f}")
        h, w = ref.shape
        pois = O.grid_pois(w, h, r, step)
        O.run_pair(ref.astype(np.float32), tar.astype(np.float32), pois, r)
        cpu = {"u": pois["p"][:, O.P_U], "v": pois["p"][:, O.P_V], "zncc": pois["r"][:, O.R_ZNCC]}
        res = C.compare_frame(cpu, {"u": got["u"], "v": got["v"], "zncc": got["zncc"]},
                              min_shared_valid=min(100, len(q) // 2))
        assert res["pass"], (r, res)


def test_batch_repeats_and_rejects_bad_jobs(dic):
    jobs = _jobs()[:3]
    qs = [dic.grid_queue(ref.shape[1], ref.shape[0], r, step) for ref, tar, r, step in jobs]
    e = dic.Engine(15)
    a = [q.copy() for q in qs]
    b = [q.copy() for q in qs]
    e.batch_process([(ref, tar, r, q) for (ref, tar, r, _), q in zip(jobs, a)])
    e.batch_process([(ref, tar, r, q) for (ref, tar, r, _), q in zip(jobs, b)])
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    ref, tar, r, _ = jobs[0]
    with pytest.raises(ValueError):
        e.batch_process([(ref, tar, 33, qs[0].copy())])
    with pytest.raises(ValueError):
        e.batch_process([(ref, tar[:-1], r, qs[0].copy())])
    with pytest.raises(ValueError):
        e.batch_process([])


def test_batch_graph_replay_on_device(dic):
    """Device-resident jobs: the second identical call captures a CUDA graph, the third
    replays it; every call gives the eager call's results."""
    torch = pytest.importorskip("torch")
    jobs = _jobs()[:4]
    dev = []
    pristine = []
    for ref, tar, r, step in jobs:
        q = dic.grid_queue(ref.shape[1], ref.shape[0], r, step)
        qd = torch.from_numpy(q.view(np.uint8).copy()).cuda()
        pristine.append(qd.clone())
        dev.append((torch.from_numpy(ref).cuda(), torch.from_numpy(tar).cuda(), r, qd))
    host = [dic.grid_queue(ref.shape[1], ref.shape[0], r, step) for ref, tar, r, step in jobs]
    e = dic.Engine(15)
    e.batch_process([(ref, tar, r, q) for (ref, tar, r, _), q in zip(jobs, host)])
    reports = []
    for call in range(3):
        for (_, _, _, qd), p in zip(dev, pristine):
            qd.copy_(p)
        reports.append(e.batch_process_device(dev))
        for (_, _, _, qd), want in zip(dev, host):
            got = qd.cpu().numpy().view(dic.POI_DTYPE)
            np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8), err_msg=f"call {call}")
    assert [r["graph"] for r in reports] == [0, 1, 1], reports
    e.set_graphs(False)
    for (_, _, _, qd), p in zip(dev, pristine):
        qd.copy_(p)
    assert e.batch_process_device(dev)["graph"] == 0


def test_autotuner_keeps_results(dic):
    """Tuned launch shapes (POIs per CTA, CTAs per SM) change no result: per-queue and
    persistent IC-GN, column and flat walks."""
    from fasticgn_gb300 import speckle
    jobs = _jobs()[:4]
    qs = [dic.grid_queue(ref.shape[1], ref.shape[0], r, max(1, step // 2)) for ref, tar, r, step in jobs]
    plain = dic.Engine(15)
    a = [q.copy() for q in qs]
    plain.batch_process([(ref, tar, r, q) for (ref, tar, r, _), q in zip(jobs, a)])
    tuned = dic.Engine(15)
    tuned.set_autotune(True)
    b = [q.copy() for q in qs]
    tuned.batch_process([(ref, tar, r, q) for (ref, tar, r, _), q in zip(jobs, b)])
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))
    t = tuned.tuning()
    assert t["batch_column_px"]["tuned"] and t["batch_column_px"]["warps_per_cta"] in (2, 4, 8), t
    assert t["batch_column_px"]["ctas_per_sm"] >= 1 and t["batch_column_px"]["ms"] > 0, t

    pr = speckle.pair_bumps(seed=90, width=512, height=512, max_disp=6.0, max_strain=0.01)
    for r in (15, 20):
        q = dic.grid_queue(512, 512, r, 4)
        e1, e2 = dic.Engine(r), dic.Engine(r)
        e2.set_autotune(True)
        out = []
        for e in (e1, e2):
            e.set_ref(pr.ref)
            e.set_tar(pr.tar)
            qq = q.copy()
            e.process_pair(qq)
            out.append(qq)
        np.testing.assert_array_equal(out[0].view(np.uint8), out[1].view(np.uint8))
        key = "icgn_column_px" if r == 15 else "icgn_pair_px"
        assert e2.tuning()[key]["tuned"] == 1, e2.tuning()

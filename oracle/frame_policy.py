"""TEST INFRASTRUCTURE: processFrame's seeding and fallback policy restated over the oracle.

Follows opencorr_cli_cuda_mvp.cpp:3024-3210 (processFrame), :560-624 (seedPoiQueueFromPrevious,
with its temporal extrapolation and :481-504 for its thresholds), :490-558 (isBadPoiForFallback, shouldReplacePoiWithFallback,
shouldTakeFrameFallbackResult, isPoiLevelFallbackCandidate), :2955-3022 (runPoiLevelFallback)
and the sequence loop's baseline rule :4244-4279.  POIs are oracle POI2D records.
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle as O

SKIP_ZNCC = 0.8
MARGIN = 0.03
TEMPORAL_MIN_STEP = np.float32(0.05)   # kTemporalSeedMinStepPx (:481)


def is_bad(z, thr=SKIP_ZNCC):
    return z != -3.0 and (not math.isfinite(z) or z < thr)


def replace_with_fallback(cur_z, fb_z):
    if not math.isfinite(fb_z) or fb_z == -3.0:
        return False
    if not math.isfinite(cur_z):
        return True
    return fb_z >= cur_z


def take_frame_fallback(skip_z, scratch_z, thr=SKIP_ZNCC):
    if skip_z == -3.0:
        return math.isfinite(scratch_z) and scratch_z != -3.0 and scratch_z >= thr
    if is_bad(skip_z, thr):
        return replace_with_fallback(skip_z, scratch_z)
    return False


def is_candidate(cur, prev, bad, thr=SKIP_ZNCC):
    if not bad:
        return False
    z = float(cur["r"][O.R_ZNCC])
    if not math.isfinite(z) or z < 0.0:
        return True
    if prev is None or prev["x"] != cur["x"] or prev["y"] != cur["y"] or not math.isfinite(float(prev["r"][O.R_ZNCC])):
        return True
    return float(prev["r"][O.R_ZNCC]) >= thr


class Solver:
    """Oracle FFTCC + IC-GN on one fixed reference and a changing target."""

    def __init__(self, ref, radius, conv=0.001, max_iter=10, threads=None):
        self.ref = np.ascontiguousarray(ref, dtype=np.float32)
        self.gx, self.gy = O.gradient(self.ref, threads)
        self.r, self.conv, self.max_iter, self.threads = radius, conv, max_iter, threads

    def set_tar(self, tar):
        self.tar = np.ascontiguousarray(tar, dtype=np.float32)
        self.coef = O.bspline_prepare(self.tar, self.threads)

    def fftcc(self, q):
        O.fftcc2d(self.ref, self.tar, q, self.r, self.threads)

    def icgn(self, q):
        O.icgn2d1(self.ref, self.gx, self.gy, self.coef, q, self.r, self.conv, self.max_iter, self.threads)


def eligible_history(p, thr=SKIP_ZNCC):
    """isEligibleTemporalSeedHistory (:499-504)."""
    u, v, z = float(p["p"][O.P_U]), float(p["p"][O.P_V]), float(p["r"][O.R_ZNCC])
    return math.isfinite(u) and math.isfinite(v) and math.isfinite(z) and z >= thr


def seed_from_previous(template, prev, prev2=None, temporal=False, max_delta=math.inf, thr=SKIP_ZNCC):
    """seedPoiQueueFromPrevious: returns (queue, POIs seeded by temporal extrapolation).  The
    extrapolation is the CPU's float arithmetic, one rounding per operation."""
    q = template.copy()
    count = 0
    f32 = np.float32
    with np.errstate(over="ignore", invalid="ignore"):
        for i in range(len(q)):
            z = float(prev["r"][i, O.R_ZNCC])
            if not math.isfinite(z) or z < 0.0:
                continue
            q["p"][i] = prev["p"][i]
            if (temporal and prev2 is not None and prev[i]["x"] == prev2[i]["x"] and prev[i]["y"] == prev2[i]["y"]
                    and prev[i]["x"] == template[i]["x"] and prev[i]["y"] == template[i]["y"]
                    and eligible_history(prev[i], thr) and eligible_history(prev2[i], thr)):
                pu, pv = f32(prev["p"][i, O.P_U]), f32(prev["p"][i, O.P_V])
                du = f32(pu - f32(prev2["p"][i, O.P_U]))
                dv = f32(pv - f32(prev2["p"][i, O.P_V]))
                nu, nv = f32(pu + du), f32(pv + dv)
                step_sq = f32(f32(du * du) + f32(dv * dv))
                if (math.isfinite(float(nu)) and math.isfinite(float(nv))
                        and step_sq >= f32(TEMPORAL_MIN_STEP * TEMPORAL_MIN_STEP)
                        and abs(float(du)) <= max_delta and abs(float(dv)) <= max_delta):
                    q["p"][i, O.P_U] = nu
                    q["p"][i, O.P_V] = nv
                    count += 1
            q["r"][i] = 0.0
            q["e"][i] = 0.0
    return q, count


def process_frame(solver, template, prev, skip, poi_fallback=True, threshold=math.inf, thr=SKIP_ZNCC,
                  prev2=None, temporal=False):
    """Returns (queue, info) as processFrame leaves them."""
    info = {"frame_fallback": False, "candidates": 0, "bad": 0, "recovered": 0, "temporal": 0}
    if not skip or prev is None:
        q = template.copy()
        solver.fftcc(q)
        solver.icgn(q)
        info["bad"] = sum(is_bad(float(z), thr) for z in q["r"][:, O.R_ZNCC])
        return q, info
    q, info["temporal"] = seed_from_previous(template, prev, prev2, temporal, float(solver.r), thr)
    solver.icgn(q)
    bad_count = 0
    cands = []
    for i in range(len(q)):
        b = is_bad(float(q["r"][i, O.R_ZNCC]), thr)
        bad_count += b
        if poi_fallback and is_candidate(q[i], prev[i], b, thr):
            cands.append(i)
    info["bad"] = bad_count
    ratio = np.float32(bad_count) / np.float32(len(q)) if len(q) else np.float32(0)
    if ratio > np.float32(threshold):
        info["frame_fallback"] = True
        scratch = template.copy()
        solver.fftcc(scratch)
        solver.icgn(scratch)
        for i in range(len(q)):
            if take_frame_fallback(float(q["r"][i, O.R_ZNCC]), float(scratch["r"][i, O.R_ZNCC]), thr):
                q[i] = scratch[i]
    elif poi_fallback and cands:
        info["candidates"] = len(cands)
        fq = np.ascontiguousarray(template[cands])
        solver.fftcc(fq)
        solver.icgn(fq)
        for k, i in enumerate(cands):
            if replace_with_fallback(float(q["r"][i, O.R_ZNCC]), float(fq["r"][k, O.R_ZNCC])):
                info["recovered"] += not is_bad(float(fq["r"][k, O.R_ZNCC]), thr)
                q[i] = fq[k]
    return q, info


def run_sequence(ref, targets, template, radius, skip=True, poi_fallback=True, threads=None, temporal=False):
    """The multi-frame loop: frame 0 from scratch sets the baseline bad ratio; later frames are
    seeded from the previous results with threshold = baseline + 0.03 (and, with temporal,
    from the two previous results); the history shifts after every frame (:4376-4377)."""
    solver = Solver(ref, radius, threads=threads)
    prev = prev2 = None
    threshold = math.inf
    out = []
    for k, tar in enumerate(targets):
        solver.set_tar(tar)
        use_skip = skip and k > 0
        q, info = process_frame(solver, template, prev if use_skip else None, use_skip, poi_fallback, threshold,
                                prev2=prev2 if use_skip else None, temporal=temporal)
        if skip and k == 0:
            threshold = float(np.float32(np.float32(info["bad"]) / np.float32(len(q))) + np.float32(MARGIN))
        out.append((q, info))
        prev2, prev = prev, q
    return out


LEARNED_MAX_ITER = 6       # IC-GN budget from a proposal seed
LEARNED_ACCEPT = 0.9       # ZNCC a proposal-seeded result must reach


def learned_policy(solver, template, seeds):
    """The learned-seed policy (no reference counterpart; the engine's enqueue_learned):
    IC-GN from the proposal's seeds with at most LEARNED_MAX_ITER iterations, then every POI
    that did not reach ZNCC LEARNED_ACCEPT (failed, NaN, or below it) is solved again from the
    template by FFTCC + IC-GN with the full budget, and that result replaces the first one.
    `seeds` holds the six first-order parameters per POI (u, ux, uy, v, vx, vy), e.g. the
    network's own output, so the oracle runs from the seeds the GPU ran from.  Returns
    (queue, number of fallback POIs)."""
    q = template.copy()
    for k, idx in enumerate((O.P_U, O.P_UX, O.P_UY, O.P_V, O.P_VX, O.P_VY)):
        q["p"][:, idx] = seeds[:, k]
    q["r"] = 0.0
    q["e"] = 0.0
    full = solver.max_iter
    solver.max_iter = min(LEARNED_MAX_ITER, full)
    try:
        solver.icgn(q)
    finally:
        solver.max_iter = full
    z = q["r"][:, O.R_ZNCC]
    with np.errstate(invalid="ignore"):
        cands = np.flatnonzero(~(z >= LEARNED_ACCEPT))
    if len(cands):
        fq = np.ascontiguousarray(template[cands])
        solver.fftcc(fq)
        solver.icgn(fq)
        q[cands] = fq
    return q, len(cands)

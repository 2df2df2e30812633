"""TEST INFRASTRUCTURE: processFrame's seeding and fallback policy restated over the oracle.

Follows opencorr_cli_cuda_mvp.cpp:3024-3210 (processFrame), :560-624 (seedPoiQueueFromPrevious,
without temporal extrapolation), :490-558 (isBadPoiForFallback, shouldReplacePoiWithFallback,
shouldTakeFrameFallbackResult, isPoiLevelFallbackCandidate), :2955-3022 (runPoiLevelFallback)
and the sequence loop's baseline rule :4244-4279.  POIs are oracle POI2D records.
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle as O

SKIP_ZNCC = 0.8
MARGIN = 0.03


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


def seed_from_previous(template, prev):
    q = template.copy()
    for i in range(len(q)):
        z = float(prev["r"][i, O.R_ZNCC])
        if not math.isfinite(z) or z < 0.0:
            continue
        q["p"][i] = prev["p"][i]
        q["r"][i] = 0.0
        q["e"][i] = 0.0
    return q


def process_frame(solver, template, prev, skip, poi_fallback=True, threshold=math.inf, thr=SKIP_ZNCC):
    """Returns (queue, info) as processFrame leaves them."""
    info = {"frame_fallback": False, "candidates": 0, "bad": 0, "recovered": 0}
    if not skip or prev is None:
        q = template.copy()
        solver.fftcc(q)
        solver.icgn(q)
        info["bad"] = sum(is_bad(float(z), thr) for z in q["r"][:, O.R_ZNCC])
        return q, info
    q = seed_from_previous(template, prev)
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


def run_sequence(ref, targets, template, radius, skip=True, poi_fallback=True, threads=None):
    """The multi-frame loop: frame 0 from scratch sets the baseline bad ratio; later frames are
    seeded from the previous results with threshold = baseline + 0.03."""
    solver = Solver(ref, radius, threads=threads)
    prev = None
    threshold = math.inf
    out = []
    for k, tar in enumerate(targets):
        solver.set_tar(tar)
        use_skip = skip and k > 0
        q, info = process_frame(solver, template, prev if use_skip else None, use_skip, poi_fallback, threshold)
        if skip and k == 0:
            threshold = float(np.float32(np.float32(info["bad"]) / np.float32(len(q))) + np.float32(MARGIN))
        out.append((q, info))
        prev = q
    return out

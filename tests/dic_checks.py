"""Shared scoring for the tests: the reference's parity checker and accuracy metrics.

``compare_frame`` restates smoke/check_cpu_gpu_parity.py:46-98 (per-frame median / p99 /
max displacement difference on POIs valid on both sides, retention and validity
disagreement); ``accuracy`` restates the per-frame metrics of
smoke/run_subpixel_accuracy_gate.py:231-289 against an exact truth.
"""
from __future__ import annotations

import math

import numpy as np


def nearest_rank(values, fraction):
    v = np.sort(np.asarray(values, dtype=np.float64))
    return float(v[max(0, math.ceil(len(v) * fraction) - 1)])


def finite_valid(u, v, z):
    return (z >= 0.0) & np.isfinite(u) & np.isfinite(v) & np.isfinite(z)


def compare_frame(cpu, gpu, median_threshold=1e-3, p99_threshold=1e-2, max_threshold=0.5,
                  min_shared_valid=100, min_valid_retention=0.95, max_validity_disagreement=0.05):
    """cpu / gpu: dicts of equal-length arrays u, v, zncc over the same POIs in the same order."""
    cv = finite_valid(cpu["u"], cpu["v"], cpu["zncc"])
    gv = finite_valid(gpu["u"], gpu["v"], gpu["zncc"])
    both = cv & gv
    lost = int((cv & ~gv).sum())
    gained = int((gv & ~cv).sum())
    n = len(cv)
    du = np.abs(cpu["u"][both] - gpu["u"][both]).astype(np.float64)
    dv = np.abs(cpu["v"][both] - gpu["v"][both]).astype(np.float64)
    res = {"shared": n, "cpu_valid": int(cv.sum()), "gpu_valid": int(gv.sum()),
           "shared_valid": int(both.sum()),
           "valid_retention": float(both.sum() / cv.sum()) if cv.sum() else 0.0,
           "validity_disagreement": (lost + gained) / n if n else 1.0,
           "cpu_valid_gpu_invalid": lost, "gpu_valid_cpu_invalid": gained, "errors": []}
    if res["shared_valid"] < min_shared_valid:
        res["errors"].append(f"shared valid POIs {res['shared_valid']} below {min_shared_valid}")
    if res["valid_retention"] < min_valid_retention:
        res["errors"].append(f"CPU-valid retention {res['valid_retention']:.4f} below {min_valid_retention}")
    if res["validity_disagreement"] > max_validity_disagreement:
        res["errors"].append(f"validity disagreement {res['validity_disagreement']:.4f}")
    if len(du):
        res.update(median_du=float(np.median(du)), median_dv=float(np.median(dv)),
                   p99_du=nearest_rank(du, .99), p99_dv=nearest_rank(dv, .99),
                   max_du=float(du.max()), max_dv=float(dv.max()))
        if max(res["median_du"], res["median_dv"]) > median_threshold:
            res["errors"].append("median displacement difference above threshold")
        if max(res["p99_du"], res["p99_dv"]) > p99_threshold:
            res["errors"].append("p99 displacement difference above threshold")
        if max(res["max_du"], res["max_dv"]) > max_threshold:
            res["errors"].append("maximum displacement difference above threshold")
    res["pass"] = not res["errors"]
    return res


def affine_truth(motion, centre, x, y):
    u0, v0, ux, uy, vx, vy = motion
    xc, yc = centre
    return u0 + ux * (x - xc) + uy * (y - yc), v0 + vx * (x - xc) + vy * (y - yc)


def accuracy(res, motion, centre, width, height, radius):
    """Per-frame metrics of the sub-pixel accuracy gate; res has x y u v ux uy vx vy zncc."""
    x = res["x"].astype(np.float64)
    y = res["y"].astype(np.float64)
    ut, vt = affine_truth(motion, centre, x, y)
    z = res["zncc"]
    valid = np.isfinite(z) & (z >= 0.0)
    measurable = ((x + ut - radius >= 2.0) & (y + vt - radius >= 2.0)
                  & (x + ut + radius < width - 3.0) & (y + vt + radius < height - 3.0))
    du = res["u"][valid] - ut[valid]
    dv = res["v"][valid] - vt[valid]
    worst = np.maximum(np.abs(du), np.abs(dv))
    grads = [res[k][valid] - t for k, t in zip(("ux", "uy", "vx", "vy"), motion[2:])]
    out = {
        "valid_ratio": float((measurable & valid).sum() / measurable.sum()),
        "valid": int(valid.sum()),
        "rmse_u": float(np.sqrt(np.mean(du ** 2))), "rmse_v": float(np.sqrt(np.mean(dv ** 2))),
        "bias_u": float(np.mean(du)), "bias_v": float(np.mean(dv)),
        "p99": nearest_rank(worst, .99), "max": float(worst.max()),
        "grad_rmse": max(float(np.sqrt(np.mean(g.astype(np.float64) ** 2))) for g in grads),
        "zncc_median": nearest_rank(z[valid], .5),
        "high_conf_wrong": int(((z[valid] >= 0.8) & (worst > 1.0)).sum()),
    }
    return out


def check_accuracy(m, limits):
    errs = []
    if m["high_conf_wrong"]:
        errs.append(f"{m['high_conf_wrong']} POIs zncc>=0.8 and >1 px off")
    if not m["valid_ratio"] >= limits["min_valid_ratio"]:
        errs.append(f"valid ratio {m['valid_ratio']:.4f}")
    for k in ("rmse_u", "rmse_v"):
        if not m[k] <= limits["max_rmse_px"]:
            errs.append(f"{k} {m[k]:.5f}")
    for k in ("bias_u", "bias_v"):
        if not abs(m[k]) <= limits["max_bias_px"]:
            errs.append(f"{k} {m[k]:.5f}")
    if not m["p99"] <= limits["max_p99_px"]:
        errs.append(f"p99 {m['p99']:.4f}")
    if not m["grad_rmse"] <= limits["max_grad_rmse"]:
        errs.append(f"grad rmse {m['grad_rmse']:.6f}")
    if not m["zncc_median"] >= limits["min_zncc_median"]:
        errs.append(f"zncc median {m['zncc_median']:.4f}")
    return errs


def oob_band(x, y, radius, width, height, dx, dy):
    """smoke/run_oob_rejection_gate.py predicted_out_of_range."""
    return ((x + dx - radius < 1.0) | (y + dy - radius < 1.0)
            | (x + dx + radius >= width - 2.0) | (y + dy + radius >= height - 2.0))


def block_relation(x, y, radius, block_x, block_y, side):
    """smoke/run_zero_texture_gate.py block_relation: 0 outside, 1 partial, 2 inside."""
    rel = np.zeros(len(x), dtype=np.int32)
    for x0 in block_x:
        x1, y1 = x0 + side - 1, block_y + side - 1
        inside = (x - radius >= x0) & (x + radius <= x1) & (y - radius >= block_y) & (y + radius <= y1)
        overlap = (x + radius >= x0) & (x - radius <= x1) & (y + radius >= block_y) & (y - radius <= y1)
        rel = np.where(inside, 2, np.where(overlap & (rel < 2), np.maximum(rel, 1), rel))
    return rel


def failure_codes(z):
    """The failure flag of each POI: its negative zncc (-3, -4, -5, or a negative incoming
    value kept by the entry test), 0 for a solved POI."""
    z = np.asarray(z)
    return np.where(np.isfinite(z) & (z < 0), z, 0)


def flags_agree(cpu, gpu, conv=1e-3):
    """Converged/failed flags of two runs over the same queue (dicts or structured arrays with
    u0, v0, zncc, and iteration / convergence where present).  Returns (fraction of POIs whose
    FFTCC seeds agree, number of POIs with the same seed and different flags, how many of those
    are iteration-cap boundary cases).  Integer FFTCC peaks may differ only on exact ties of the
    correlation map; from the same seed the flags must be identical, except where both runs
    used the whole iteration budget and the last step's size lies within a factor of two of the
    criterion: whether such a POI ends converged (0) or at the cap (-4) is decided by float
    rounding of a slowly converging iteration, on either side."""
    same = (np.asarray(cpu["u0"]) == np.asarray(gpu["u0"])) & (np.asarray(cpu["v0"]) == np.asarray(gpu["v0"]))
    fc, fg = failure_codes(cpu["zncc"]), failure_codes(gpu["zncc"])
    diff = (fc != fg) & same
    boundary = np.zeros(len(fc), dtype=bool)
    if all(k in cpu and k in gpu for k in ("iteration", "convergence")):
        ic, ig = np.asarray(cpu["iteration"]), np.asarray(gpu["iteration"])
        cap = max(float(np.nanmax(ic)) if len(ic) else 0.0, float(np.nanmax(ig)) if len(ig) else 0.0)
        cc, cg = np.asarray(cpu["convergence"]), np.asarray(gpu["convergence"])
        with np.errstate(invalid="ignore"):
            boundary = ((ic == cap) & (ig == cap) & np.isin(fc, (0, -4)) & np.isin(fg, (0, -4))
                        & (cc >= 0.5 * conv) & (cc <= 2 * conv) & (cg >= 0.5 * conv) & (cg <= 2 * conv))
    return float(same.mean()) if len(same) else 1.0, int(diff.sum()), int((diff & boundary).sum())


def flag_differences(cpu, gpu, limit=8):
    """(cpu code, gpu code, cpu iterations, gpu iterations) of up to `limit` POIs whose
    failure flags differ, for messages."""
    fc, fg = failure_codes(cpu["zncc"]), failure_codes(gpu["zncc"])
    idx = np.flatnonzero(fc != fg)[:limit]
    it_c = cpu.get("iteration", np.full(len(fc), np.nan))
    it_g = gpu.get("iteration", np.full(len(fg), np.nan))
    return [(float(fc[i]), float(fg[i]), float(it_c[i]), float(it_g[i])) for i in idx]


def assert_flags_agree(cpu, gpu, min_same_seed=0.999, max_boundary=1e-3):
    """Same-seed flags identical, up to iteration-cap boundary cases (flags_agree) on at most
    `max_boundary` of the POIs."""
    same, bad, boundary = flags_agree(cpu, gpu)
    assert same >= min_same_seed, f"FFTCC seeds agree on {same:.5f} of the POIs"
    n = max(len(np.asarray(cpu["zncc"])), 1)
    assert bad == boundary and boundary <= max_boundary * n, (
        f"{bad} POIs with the same seed have different failure flags, {boundary} of them at the iteration cap "
        f"(cpu code, gpu code, cpu iterations, gpu iterations): {flag_differences(cpu, gpu)}")

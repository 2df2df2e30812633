"""CPU tests of the oracle: pinned to the reference's golden cases and known answers.

The oracle (oracle/dic_oracle.cpp) restates OpenCorr's CPU path; the reference itself cannot
be built here (Eigen, OpenCV and FFTW are absent), so it is pinned by
  * the sub-pixel accuracy gate's cases and limits (smoke/run_subpixel_accuracy_gate.py),
  * whole-pixel shift sequences with exact truth (smoke/generate_synthetic_dic.py),
  * the closed-form out-of-range band (smoke/run_oob_rejection_gate.py),
  * the zero-texture rule for the CPU backend (smoke/run_zero_texture_gate.py: -5 inside a
    constant block, exact self-match outside),
  * its own FFT against numpy's DFT.
"""
import json

import numpy as np
import pytest

import dic_checks as C


def run_oracle_pair(O, ref, tar, radius, step, threads=None):
    h, w = ref.shape
    pois = O.grid_pois(w, h, radius, step)
    O.run_pair(ref.astype(np.float32), tar.astype(np.float32), pois, radius, threads=threads)
    return pois


def as_fields(O, pois):
    p, r = pois["p"], pois["r"]
    return {"x": pois["x"], "y": pois["y"], "u": p[:, O.P_U], "v": p[:, O.P_V], "ux": p[:, O.P_UX],
            "uy": p[:, O.P_UY], "vx": p[:, O.P_VX], "vy": p[:, O.P_VY], "zncc": r[:, O.R_ZNCC],
            "iteration": r[:, O.R_ITER]}


@pytest.mark.parametrize("case", ["s15", "s15_lowsnr", "s63"])
def test_oracle_subpixel_accuracy_gate(oracle_mod, golden, case):
    """Every frame of the gate's cases meets its accuracy limits (single-pair FFTCC + IC-GN)."""
    O = oracle_mod
    g = golden(case)
    limits = json.loads(str(g["limits"]))
    ref, radius, grid = g["ref"], int(g["radius"]), int(g["grid"])
    h, w = ref.shape
    for k, motion in enumerate(g["motions"]):
        res = as_fields(O, run_oracle_pair(O, ref, g["tars"][k], radius, grid))
        m = C.accuracy(res, motion, g["centre"], w, h, radius)
        errs = C.check_accuracy(m, limits)
        assert not errs, f"{case} frame {k}: {errs} {m}"


def test_oracle_whole_pixel_shifts_exact(oracle_mod, golden):
    """A noise-free whole-pixel shift is recovered exactly (u = dx, v = dy, zncc 1)."""
    O = oracle_mod
    g = golden("shift")
    ref, radius = g["ref"], int(g["radius"])
    h, w = ref.shape
    for (dx, dy), tar in zip(g["shifts"], g["tars"]):
        res = as_fields(O, run_oracle_pair(O, ref, tar, radius, 1))
        x, y = res["x"], res["y"]
        # subsets whose target footprint stays inside the unfilled part of the shifted image
        inside = (x - radius - 2 >= dx + 1) & (y - radius - 2 >= dy + 1) & \
                 (x + dx + radius + 3 < w) & (y + dy + radius + 3 < h)
        assert inside.sum() > 100
        assert np.all(np.abs(res["u"][inside] - dx) <= 1e-4)
        assert np.all(np.abs(res["v"][inside] - dy) <= 1e-4)
        assert np.all(res["zncc"][inside] >= 0.9999)


def test_oracle_oob_band(oracle_mod, golden):
    """Every POI the 10-px shift pushes off the image is -3; the rest stay valid."""
    O = oracle_mod
    g = golden("oob")
    ref, tar, radius, shift = g["ref"], g["tar"], int(g["radius"]), int(g["shift"])
    h, w = ref.shape
    pois = O.grid_pois(w, h, radius, 1)
    # seed with the known shift, as the gate's FFTCC does for interior POIs
    pois["p"][:, O.P_U] = shift
    gx, gy = O.gradient(ref.astype(np.float32))
    coef = O.bspline_prepare(tar.astype(np.float32))
    O.icgn2d1(ref.astype(np.float32), gx, gy, coef, pois, radius)
    res = as_fields(O, pois)
    band = C.oob_band(res["x"], res["y"], radius, w, h, shift, 0)
    assert band.sum() > 0 and (~band).sum() > 0
    assert np.all(res["zncc"][band] == -3.0)
    # the incoming guess is kept on rejection
    assert np.all(res["u"][band] == shift)
    assert np.all(res["zncc"][~band] != -3.0)


def test_oracle_zero_texture(oracle_mod, golden):
    """CPU rule: -5 with u = v = 0 inside a constant block; exact self-match outside."""
    O = oracle_mod
    g = golden("zero_texture")
    ref, radius = g["ref"], int(g["radius"])
    h, w = ref.shape
    res = as_fields(O, run_oracle_pair(O, ref, ref, radius, 1))
    rel = C.block_relation(res["x"], res["y"], radius, g["block_x"], int(g["block_y"]), int(g["block_side"]))
    inside, outside = rel == 2, rel == 0
    assert inside.sum() > 0
    assert np.all(res["zncc"][inside] == -5.0)
    assert np.all(res["u"][inside] == 0.0) and np.all(res["v"][inside] == 0.0)
    assert np.all(res["zncc"][outside] == 1.0)
    assert np.all(np.abs(res["u"][outside]) <= 1e-4) and np.all(np.abs(res["v"][outside]) <= 1e-4)


def test_oracle_fft_matches_dft(oracle_mod):
    """The oracle's own FFT gives the unnormalised correlation map FFTW's r2c/c2r pair does."""
    O = oracle_mod
    rng = np.random.default_rng(7)
    for radius in (5, 12, 15):
        m = 2 * radius
        ref = rng.uniform(0, 255, (64, 64)).astype(np.float32)
        tar = np.roll(ref, (2, -3), axis=(0, 1)) + rng.normal(0, 1, ref.shape).astype(np.float32)
        cmap = O.fftcc2d_map(ref, tar, radius, 32.0, 32.0)
        rs = ref[32 - radius:32 + radius, 32 - radius:32 + radius].astype(np.float64)
        ts = tar[32 - radius:32 + radius, 32 - radius:32 + radius].astype(np.float64)
        rs -= rs.mean()
        ts -= ts.mean()
        want = np.fft.ifft2(np.conj(np.fft.fft2(rs)) * np.fft.fft2(ts)).real * m * m
        np.testing.assert_allclose(cmap, want, rtol=0, atol=2e-5 * np.abs(want).max())


def test_oracle_fftcc_integer_shift(oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(3)
    ref = rng.uniform(0, 255, (96, 96)).astype(np.float32)
    for dx, dy in [(0, 0), (3, -2), (-7, 5), (15, 0)]:
        tar = np.roll(ref, (dy, dx), axis=(0, 1))
        pois = O.make_pois([48.0], [48.0])
        O.fftcc2d(ref, tar, pois, 15)
        assert pois["p"][0, O.P_U] == dx and pois["p"][0, O.P_V] == dy
        # windows overlap only partly once shifted, so zncc is 1 only for the zero shift
        if dx == 0 and dy == 0:
            assert abs(pois["r"][0, O.R_ZNCC] - 1.0) < 1e-5
        else:
            assert 0.3 < pois["r"][0, O.R_ZNCC] < 1.0


def test_oracle_bspline_integer_nodes(oracle_mod):
    """At integer positions the table's c[0][0] term returns the pixel value exactly."""
    O = oracle_mod
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (20, 24)).astype(np.float32)
    coef = O.bspline_prepare(img)
    for y in range(1, 17):
        for x in range(1, 21):
            assert O.bspline_value(coef, float(x), float(y)) == img[y, x]
    assert O.bspline_value(coef, 0.5, 5.0) == -1.0      # x < 1
    assert O.bspline_value(coef, 5.0, 18.0) == -1.0     # y >= h - 2


def test_policy_temporal_seed_rules(oracle_mod):
    """seedPoiQueueFromPrevious's temporal extrapolation (:594-616) in the restated policy:
    prev + (prev - prev_prev) for u and v only where both results are eligible (finite, zncc
    >= 0.8) at the template's location, the step is >= 0.05 px and each component's step is
    within the subset radius."""
    O = oracle_mod
    from oracle import frame_policy as FP
    n = 8
    tmpl = np.zeros(n, dtype=O.POI2D_DTYPE)
    tmpl["x"] = np.arange(n) * 10.0 + 20.0
    tmpl["y"] = 30.0
    prev, prev2 = tmpl.copy(), tmpl.copy()
    prev["r"][:, O.R_ZNCC] = 0.95
    prev2["r"][:, O.R_ZNCC] = 0.95
    prev["p"][:, O.P_U] = 1.0
    prev["p"][:, O.P_V] = -0.5
    prev["p"][:, O.P_UX] = 0.001
    prev2["p"][:, O.P_U] = 0.8          # step (0.2, 0.1): extrapolated to (1.2, -0.4)
    prev2["p"][:, O.P_V] = -0.6
    prev2["p"][1, O.P_U] = 0.99         # step 0.01 px: below 0.05, not extrapolated
    prev2["p"][1, O.P_V] = -0.5
    prev2["p"][2, O.P_U] = -20.0        # |du| = 21 > radius 15
    prev2["r"][3, O.R_ZNCC] = 0.7       # history below 0.8
    prev["r"][4, O.R_ZNCC] = np.nan     # invalid previous result: template seed, nothing copied
    prev2["x"][5] += 1.0                # another location
    prev["p"][6, O.P_V] = np.inf        # non-finite previous v
    q, count = FP.seed_from_previous(tmpl, prev, prev2, temporal=True, max_delta=15.0)
    assert count == 2                   # POIs 0 and 7
    for i in (0, 7):
        assert q["p"][i, O.P_U] == np.float32(np.float32(1.0) + np.float32(np.float32(1.0) - np.float32(0.8)))
        assert q["p"][i, O.P_V] == np.float32(np.float32(-0.5) + np.float32(np.float32(-0.5) - np.float32(-0.6)))
        assert q["p"][i, O.P_UX] == np.float32(0.001)   # the other parameters are copied as they were
    for i in (1, 2, 3, 5, 6):
        assert q["p"][i, O.P_U] == np.float32(1.0)
    assert q["p"][4, O.P_U] == 0.0 and np.all(q["r"][:, O.R_ZNCC] == 0.0)
    q0, c0 = FP.seed_from_previous(tmpl, prev, prev2, temporal=False)
    assert c0 == 0 and q0["p"][0, O.P_U] == np.float32(1.0)


def test_policy_learned_seed_fallback(oracle_mod):
    """The restated learned-seed policy (oracle/frame_policy.learned_policy): POIs whose seeds
    IC-GN confirms within 6 iterations keep that result; POIs whose seed is far off (the 6-
    iteration budget runs out, the result leaves the range, or ZNCC ends below 0.9) are solved
    again from the template by FFTCC + IC-GN, which then equals the plain FFTCC path."""
    O = oracle_mod
    from fasticgn_gb300 import speckle
    from oracle import frame_policy as FP
    pr = speckle.pair_affine(seed=21, width=192, height=160)
    ref, tar = pr.ref.astype(np.float32), pr.tar.astype(np.float32)
    tmpl = O.grid_pois(192, 160, 12, 9)
    plain = tmpl.copy()
    solver = FP.Solver(ref, 12)
    solver.set_tar(tar)
    solver.fftcc(plain)
    solver.icgn(plain)
    ok = plain["r"][:, O.R_ZNCC] >= 0.9
    assert ok.mean() > 0.8
    seeds = np.stack([plain["p"][:, k] for k in (O.P_U, O.P_UX, O.P_UY, O.P_V, O.P_VX, O.P_VY)], axis=1)
    seeds[~ok] = 0.0
    bad = np.zeros(len(tmpl), dtype=bool)
    bad[::3] = True                       # a third of the seeds 9 px off: beyond what IC-GN recovers
    seeds[bad, 0] += 9.0
    q, fallbacks = FP.learned_policy(solver, tmpl, seeds.astype(np.float32))
    z = q["r"][:, O.R_ZNCC]
    good = ok & ~bad
    # converged seeds: confirmed in a few iterations, at the plain path's solution
    assert np.all(q["r"][good, O.R_ITER] <= 3)
    assert np.max(np.abs(q["p"][good, O.P_U] - plain["p"][good, O.P_U])) < 1e-3
    # the displaced seeds fell back, and their results are the plain path's, bit for bit
    fb = q["r"][:, O.R_U0] == np.round(q["r"][:, O.R_U0])
    assert fallbacks >= bad.sum() * 0.9 and np.all(fb[bad & ok])
    np.testing.assert_array_equal(q[bad & ok].view(np.uint8), plain[bad & ok].view(np.uint8))
    assert np.all((z[ok] >= 0.9))


def test_flag_agreement_rule():
    """The flag rule the GPU parity tests apply (tests/dic_checks.py): from the same seed the
    failure codes must be identical, except for POIs that used the whole iteration budget on
    both sides with a last step within a factor of two of the criterion (0 against -4)."""
    n = 2000
    cpu = {"u0": np.zeros(n, np.float32), "v0": np.zeros(n, np.float32), "zncc": np.full(n, 0.95, np.float32),
           "iteration": np.full(n, 4.0, np.float32), "convergence": np.full(n, 2e-4, np.float32)}
    gpu = {k: v.copy() for k, v in cpu.items()}
    assert C.flags_agree(cpu, gpu) == (1.0, 0, 0)
    # a cap-boundary flip: both at 10 iterations, last steps 0.9e-3 and 1.1e-3
    for d, z, c in ((cpu, 0.97, 0.9e-3), (gpu, -4.0, 1.1e-3)):
        d["iteration"][7] = 10.0
        d["zncc"][7] = z
        d["convergence"][7] = c
    assert C.flags_agree(cpu, gpu) == (1.0, 1, 1)
    C.assert_flags_agree(cpu, gpu)
    # a flip away from the cap is a parity failure
    gpu["zncc"][9] = -5.0
    assert C.flags_agree(cpu, gpu) == (1.0, 2, 1)
    with pytest.raises(AssertionError):
        C.assert_flags_agree(cpu, gpu)
    # different FFTCC seeds are not compared
    gpu["zncc"][9] = 0.95
    gpu["u0"][11] = 1.0
    gpu["zncc"][11] = -3.0
    assert C.flags_agree(cpu, gpu)[1:] == (1, 1)

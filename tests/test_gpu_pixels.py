"""GPU tests of pixel sampling (DIC_SAMPLE_PIXELS, k_icgn_px): IC-GN evaluates the bicubic
interpolant from the 4 x 4 pixels around each sample, with each POI's window staged in shared
memory (TMA where the row pitch is a multiple of 16 bytes, warp copies otherwise).

* Every launch form -- windows staged or read from the global plane, 2/4/8 warps per CTA,
  under the autotuner -- gives the same bits: a sample outside its window reads the global
  plane, and both hold the same floats.
* Against the coefficient-table sampling (BicubicBspline::compute's polynomial, per texel)
  the results differ by float rounding only, and the flags agree.
* Against the CPU oracle the parity gate holds and same-seed flags agree (the general
  parity tests run this mode too, as it is the default).
* A window copy that never arrives ends in the bounded wait and a DIC_ERR_CUDA error.
"""
import numpy as np
import pytest

import dic_checks as C

pytestmark = pytest.mark.gpu


def solve(dic, ref, tar, radius, step, sampling=None, shape=None, autotune=False):
    h, w = ref.shape
    q = dic.grid_queue(w, h, radius, step)
    e = dic.Engine(radius)
    if sampling is not None:
        e.set_sampling(sampling)
    if shape is not None:
        e.set_launch_shape(3, **shape)
    e.set_autotune(autotune)
    e.set_ref(ref)
    e.set_tar(tar)
    e.process_pair(q)
    st, tun = e.stats(), e.tuning()
    e.close()
    return q, st, tun


@pytest.mark.parametrize("radius,step,width", [(15, 4, 384), (10, 3, 320), (7, 2, 256), (12, 5, 382), (3, 6, 200)])
def test_pixel_forms_agree_bit_for_bit(dic, radius, step, width):
    """Staged (TMA, or warp copies for the 382-wide image; tile 2 always by warp copies) and
    unstaged windows, every CTA width: identical records.  Displacements up to 9 px with 2 % strain put some updates
    outside their windows (global reads inside a staged solve)."""
    from fasticgn_gb300 import speckle
    pr = speckle.pair_bumps(seed=200 + radius, width=width, height=300, max_disp=9.0, max_strain=0.02)
    want, st0, _ = solve(dic, pr.ref, pr.tar, radius, step, shape=dict(warps_per_cta=4, tile=1))
    for warps in (2, 4, 8):
        for tile in (0, 1, 2):
            got, st, tun = solve(dic, pr.ref, pr.tar, radius, step, shape=dict(warps_per_cta=warps, tile=tile))
            assert tun["icgn_column_px"]["warps_per_cta"] == warps and tun["icgn_column_px"]["tile"] == tile
            np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8), err_msg=f"{warps} {tile}")
            assert st["icgn_iterations"] == st0["icgn_iterations"]
    got, _, tun = solve(dic, pr.ref, pr.tar, radius, step, autotune=True)
    np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8))
    if radius >= 10:
        assert (want["zncc"] >= 0).mean() > 0.9
        assert tun["icgn_column_px"]["tuned"] == 1 and tun["icgn_column_px"]["ms"] > 0, tun


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.float32])
def test_pixels_match_table_and_oracle(dic, oracle_mod, dtype):
    O = oracle_mod
    from fasticgn_gb300 import speckle
    pr = speckle.pair_bumps(seed=77, width=512, height=448, max_disp=10.0, max_strain=0.02)
    scale = {np.uint8: 1, np.uint16: 16, np.float32: 1}[dtype]
    ref = (pr.ref.astype(np.float32) * scale).astype(dtype)
    tar = (pr.tar.astype(np.float32) * scale).astype(dtype)
    if dtype == np.float32:
        ref = ref + np.float32(0.25)
        tar = tar + np.float32(0.25)
    px, st_p, _ = solve(dic, ref, tar, 15, 4)
    tb, st_t, _ = solve(dic, ref, tar, 15, 4, sampling=dic._lib.DIC_SAMPLE_TABLE)
    ok = (px["zncc"] >= 0) & (tb["zncc"] >= 0)
    assert ok.mean() > 0.95
    assert np.abs(px["u"] - tb["u"])[ok].max() <= 1e-3 and np.abs(px["v"] - tb["v"])[ok].max() <= 1e-3
    assert np.median(np.abs(px["u"] - tb["u"])[ok]) <= 1e-5
    assert (C.failure_codes(px["zncc"]) == C.failure_codes(tb["zncc"])).mean() >= 0.999
    assert st_p["ms_prepare_tar"] >= 0
    oq = O.grid_pois(ref.shape[1], ref.shape[0], 15, 4)
    O.run_pair(ref.astype(np.float32), tar.astype(np.float32), oq, 15)
    cpu = {"u": oq["p"][:, O.P_U], "v": oq["p"][:, O.P_V], "zncc": oq["r"][:, O.R_ZNCC], "u0": oq["r"][:, O.R_U0],
           "v0": oq["r"][:, O.R_V0], "iteration": oq["r"][:, O.R_ITER], "convergence": oq["r"][:, O.R_CONV]}
    gpu = {k: px[k] for k in ("u", "v", "zncc", "u0", "v0", "iteration", "convergence")}
    res = C.compare_frame(cpu, gpu)
    assert res["pass"], res
    C.assert_flags_agree(cpu, gpu)


def test_sampling_switch_rebuilds_the_table(dic):
    """Switching to table sampling after a pixel solve on the same target builds the table
    then (the pixel path does not), and each mode repeats its own results."""
    from fasticgn_gb300 import speckle
    pr = speckle.pair_bumps(seed=5, width=320, height=320, max_disp=5.0, max_strain=0.01)
    q0 = dic.grid_queue(320, 320, 15, 6)
    e = dic.Engine(15)
    e.set_ref(pr.ref)
    e.set_tar(pr.tar)
    runs = []
    for mode in (dic._lib.DIC_SAMPLE_PIXELS, dic._lib.DIC_SAMPLE_TABLE, dic._lib.DIC_SAMPLE_PIXELS,
                 dic._lib.DIC_SAMPLE_TABLE):
        e.set_sampling(mode)
        q = q0.copy()
        e.process_pair(q)
        runs.append(q)
    e.close()
    np.testing.assert_array_equal(runs[0].view(np.uint8), runs[2].view(np.uint8))
    np.testing.assert_array_equal(runs[1].view(np.uint8), runs[3].view(np.uint8))
    want, _, _ = solve(dic, pr.ref, pr.tar, 15, 6, sampling=dic._lib.DIC_SAMPLE_TABLE)
    np.testing.assert_array_equal(runs[1].view(np.uint8), want.view(np.uint8))
    with pytest.raises(ValueError):
        dic.Engine(15).set_sampling(2)


def test_pixel_window_timeout_is_reported(dic, monkeypatch):
    """A window copy that never arrives (DIC_TEST_WAIT_FAULT arms the wait and skips the
    copy) ends in the bounded wait: DIC_ERR_CUDA naming the copy, nothing faults, and the
    context then solves the pair normally."""
    from fasticgn_gb300 import speckle, _lib
    pr = speckle.pair_bumps(seed=9, width=320, height=288, max_disp=4.0, max_strain=0.01)
    want, _, _ = solve(dic, pr.ref, pr.tar, 15, 4, shape=dict(warps_per_cta=4, tile=1))
    monkeypatch.setenv("DIC_TEST_WAIT_FAULT", "1")
    e = dic.Engine(15)
    monkeypatch.delenv("DIC_TEST_WAIT_FAULT")
    e.set_launch_shape(3, warps_per_cta=4, ctas_per_sm=0, tile=1)
    e.set_autotune(False)
    e.set_ref(pr.ref)
    e.set_tar(pr.tar)
    q = dic.grid_queue(320, 288, 15, 4)
    with pytest.raises(_lib.DicError) as info:
        e.process_pair(q)
    assert info.value.code == _lib.DIC_ERR_CUDA and "TMA tile copy" in str(info.value)
    e.close()
    got, _, _ = solve(dic, pr.ref, pr.tar, 15, 4, shape=dict(warps_per_cta=4, tile=1))
    np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8))

"""GPU tests of the TMA-staged IC-GN (k_icgn_tile, table sampling): each POI's result, iteration count and
flags are bit-identical to the gather form's, whether its chunk's block fits the tile (texels
from shared memory), partly fits (texels outside it from the global table) or does not fit at
all (the whole chunk from the global table), also inside a graph-captured sequence frame and
under the autotuner.  The tile form always evaluates the full bicubic polynomial, while the
gather form takes the first (integer-translation) iteration of every FFTCC-seeded POI from
the lattice plane, so these comparisons also show that the lattice samples are exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def solve(dic, pr, radius, step, tile=None, autotune=False):
    q = dic.grid_queue(pr.ref.shape[1], pr.ref.shape[0], radius, step)
    e = dic.Engine(radius)
    e.set_sampling(dic._lib.DIC_SAMPLE_TABLE)
    if tile is not None:
        e.set_launch_shape(True, tile=tile)
    e.set_autotune(autotune)
    e.set_ref(pr.ref)
    e.set_tar(pr.tar)
    e.process_pair(q)
    st = e.stats()
    tun = e.tuning()
    e.close()
    return q, st, tun


@pytest.mark.parametrize("radius,step", [(15, 4), (10, 3), (7, 2), (15, 9), (12, 16)])
def test_tile_forms_equal_gather(dic, radius, step):
    from fasticgn_gb300 import speckle
    pr = speckle.pair_bumps(seed=70 + radius, width=384, height=320, max_disp=8.0, max_strain=0.02)
    want, st0, _ = solve(dic, pr, radius, step)
    for tile in (1, 2):
        got, st, tun = solve(dic, pr, radius, step, tile=tile)
        assert tun["icgn_column"]["tile"] == tile
        np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8), err_msg=f"tile {tile}")
        assert st["icgn_iterations"] == st0["icgn_iterations"]
    if radius >= 10:   # a 14 px FFTCC window (r 7) misses many of the 8 px displacements
        assert (want["zncc"] >= 0).mean() > 0.9


def test_tile_form_in_sequence_graph(dic):
    from fasticgn_gb300 import speckle
    ref, frames = speckle.stream_frames(width=320, height=288, frames=200, which=[0, 1, 2, 3])
    tmpl = dic.grid_queue(320, 288, 15, 5)
    outs = []
    for tile in (None, 1):
        e = dic.Engine(15)
        e.set_sampling(dic._lib.DIC_SAMPLE_TABLE)
        e.set_graphs(True)
        if tile:
            e.set_launch_shape(True, tile=tile)
        e.set_ref(ref)
        e.sequence_begin(tmpl)
        got = []
        for _, tar, _ in frames:
            res = np.zeros_like(tmpl)
            e.sequence_frame(tar, res)
            got.append(res)
        e.close()
        outs.append(got)
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))


def test_autotuner_times_tile_forms(dic):
    from fasticgn_gb300 import speckle
    pr = speckle.pair_bumps(seed=5, width=512, height=512, max_disp=6.0, max_strain=0.01)
    want, _, _ = solve(dic, pr, 15, 4)
    got, _, tun = solve(dic, pr, 15, 4, autotune=True)
    np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8))
    t = tun["icgn_column"]
    assert t["tuned"] == 1 and t["tile"] in (0, 1, 2) and t["ms"] > 0, t


def test_launch_shape_arguments(dic):
    e = dic.Engine(15)
    for kw in (dict(walk=1, tile=3), dict(walk=0, tile=1), dict(walk=2, tile=1),
               dict(walk=1, warps_per_cta=3), dict(walk=1, ctas_per_sm=-1), dict(walk=5), dict(walk=3, tile=3),
               dict(walk=4, tile=3), dict(walk=3, warps_per_poi=2), dict(walk=4, warps_per_poi=3),
               dict(walk=1, warps_per_poi=2), dict(walk=2, warps_per_poi=3)):
        with pytest.raises((ValueError, RuntimeError)):
            e.set_launch_shape(**kw)
    e.set_launch_shape(True, warps_per_cta=2, ctas_per_sm=0)
    assert e.tuning()["icgn_column"]["warps_per_cta"] == 2 and e.tuning()["icgn_column"]["tile"] == 0
    e.set_launch_shape(2, warps_per_cta=8, ctas_per_sm=4, warps_per_poi=2)
    assert e.tuning()["icgn_pair"]["warps_per_poi"] == 2 and e.tuning()["icgn_pair"]["warps_per_cta"] == 8
    e.set_launch_shape(4, warps_per_cta=2, ctas_per_sm=0, tile=2, warps_per_poi=2)
    t = e.tuning()["icgn_pair_px"]
    assert t["warps_per_poi"] == 2 and t["warps_per_cta"] == 2 and t["tile"] == 2, t
    e.close()


def test_tile_copy_timeout_is_reported(dic, monkeypatch):
    """A TMA copy that never arrives (the DIC_TEST_WAIT_FAULT hook arms the wait and skips the
    copy) ends in the kernel's bounded wait: the call fails with DIC_ERR_CUDA naming the tile
    copy, nothing faults, and the same context then solves the pair normally."""
    from fasticgn_gb300 import speckle, _lib
    pr = speckle.pair_bumps(seed=9, width=320, height=288, max_disp=4.0, max_strain=0.01)
    want, _, _ = solve(dic, pr, 15, 4, tile=1)
    monkeypatch.setenv("DIC_TEST_WAIT_FAULT", "1")
    e = dic.Engine(15)
    monkeypatch.delenv("DIC_TEST_WAIT_FAULT")
    e.set_sampling(_lib.DIC_SAMPLE_TABLE)
    e.set_launch_shape(True, tile=1)
    e.set_autotune(False)
    e.set_ref(pr.ref)
    e.set_tar(pr.tar)
    q = dic.grid_queue(320, 288, 15, 4)
    with pytest.raises(_lib.DicError) as info:
        e.process_pair(q)
    assert info.value.code == _lib.DIC_ERR_CUDA and "TMA tile copy" in str(info.value)
    e.close()
    got, _, _ = solve(dic, pr, 15, 4, tile=1)
    np.testing.assert_array_equal(got.view(np.uint8), want.view(np.uint8))


def test_lattice_samples_equal_the_polynomial(dic, oracle_mod):
    """IC-GN from integer-translation seeds (the FFTCC seeds) reads its first iteration's samples
    from the lattice plane; the oracle evaluates the full polynomial at those points.  One
    iteration from a whole-pixel shift gives the CPU's flags, displacement and ZNCC to within
    the rounding of the single-pass sums."""
    O = oracle_mod
    from fasticgn_gb300 import speckle
    pr = speckle.pair_affine(seed=12, width=256, height=224)
    ref = pr.ref
    tar = np.zeros_like(ref)
    tar[:, 3:] = ref[:, :-3]            # a whole-pixel shift of 3 px in x
    q = dic.grid_queue(256, 224, 12, 5)
    q["u"] = 3.0
    oq = O.make_pois(q["x"], q["y"])
    oq["p"][:, O.P_U] = 3.0
    icgn = dic.ICGN2D1(12, 12, 0.001, 1)           # one iteration: the lattice iteration alone
    icgn.setImages(ref, tar)
    icgn.compute(q)
    r32, t32 = ref.astype(np.float32), tar.astype(np.float32)
    gx, gy = O.gradient(r32)
    O.icgn2d1(r32, gx, gy, O.bspline_prepare(t32), oq, 12, 0.001, 1)
    inside = (q["x"] - 12 - 2 > 3) & (q["zncc"] >= 0)
    assert inside.sum() > 100
    cz = oq["r"][:, O.R_ZNCC]
    assert np.array_equal(C_failure(q["zncc"]), C_failure(cz))
    np.testing.assert_allclose(q["u"][inside], oq["p"][inside, O.P_U], atol=2e-5)
    np.testing.assert_allclose(q["zncc"][inside], cz[inside], atol=2e-6)


def C_failure(z):
    return np.where(np.isfinite(z) & (z < 0), z, 0)

"""The pair walk (subsets of 33 to 64 columns, subset radius 16 to 31): two column classes
(columns 0-31 and 32 on), each reduced on its own and added in class order, walked by one
or two warps per POI, under either sampling of the target (the coefficient table, walk 2;
the pixels with each POI's window staged in shared memory, walk 4, the default).

* within a sampling mode every launch shape (one or two warps per POI, 2 / 4 / 8 warps per
  CTA, grid or persistent; for pixels the window by TMA, by warp copies or not staged)
  gives the same bytes, and the autotuner changes nothing;
* same-seed IC-GN against the CPU oracle within the reference parity gate, with identical
  failure flags and iteration counts, in both modes; pixels and table agree to float rounding;
* the exact self-match of the per-POI prep and the IC-GN sums: a target equal to the
  reference gives zncc == 1 exactly on every textured subset.
"""
import numpy as np
import pytest

import dic_checks as C

pytestmark = pytest.mark.gpu

SHAPES = [dict(warps_per_cta=4, ctas_per_sm=0, warps_per_poi=1), dict(warps_per_cta=4, ctas_per_sm=0, warps_per_poi=2),
          dict(warps_per_cta=2, ctas_per_sm=16, warps_per_poi=1), dict(warps_per_cta=8, ctas_per_sm=4, warps_per_poi=2),
          dict(warps_per_cta=2, ctas_per_sm=16, warps_per_poi=2), dict(warps_per_cta=8, ctas_per_sm=0, warps_per_poi=1)]
# pixel sampling (walk 4): tile 1 windows by TMA, 2 by warp copies, 0 none; ctas_per_sm 0 = full occupancy
SHAPES_PX = [dict(warps_per_cta=4, ctas_per_sm=0, warps_per_poi=2, tile=1), dict(warps_per_cta=4, ctas_per_sm=0, warps_per_poi=1, tile=1),
             dict(warps_per_cta=2, ctas_per_sm=0, warps_per_poi=2, tile=0), dict(warps_per_cta=8, ctas_per_sm=0, warps_per_poi=1, tile=0),
             dict(warps_per_cta=2, ctas_per_sm=0, warps_per_poi=2, tile=2), dict(warps_per_cta=8, ctas_per_sm=0, warps_per_poi=2, tile=1),
             dict(warps_per_cta=8, ctas_per_sm=0, warps_per_poi=2, tile=2), dict(warps_per_cta=2, ctas_per_sm=3, warps_per_poi=1, tile=1)]


def _engine(dic, radius, pixels):
    from fasticgn_gb300 import _lib
    e = dic.Engine(radius)
    if not pixels:
        e.set_sampling(_lib.DIC_SAMPLE_TABLE)
    return e


@pytest.mark.parametrize("pixels", [False, True])
@pytest.mark.parametrize("radius", [16, 20, 25, 31])
def test_pair_walk_shapes_give_the_same_bytes(dic, radius, pixels):
    """Displacements up to 5 px with 1 % strain: some updates leave their window (global-plane
    reads inside a staged solve)."""
    from fasticgn_gb300 import speckle
    pr = speckle.pair_bumps(seed=40 + radius, width=416, height=384, max_disp=5.0, max_strain=0.01)
    walk, key, shapes = (4, "icgn_pair_px", SHAPES_PX) if pixels else (2, "icgn_pair", SHAPES)
    outs = []
    for sh in shapes:
        with _engine(dic, radius, pixels) as e:
            e.set_launch_shape(walk, **sh)
            e.set_ref(pr.ref)
            e.set_tar(pr.tar)
            q = dic.grid_queue(416, 384, radius, 5)
            e.process_pair(q)
            t = e.tuning()[key]
            assert t["warps_per_poi"] == sh["warps_per_poi"] and t["tile"] == sh.get("tile", 0), t
        outs.append(q)
    ok = outs[0]["zncc"] >= 0
    assert ok.mean() > 0.9
    for sh, q in zip(shapes[1:], outs[1:]):
        assert q.tobytes() == outs[0].tobytes(), sh
    with _engine(dic, radius, pixels) as e:
        e.set_autotune(True)
        e.set_ref(pr.ref)
        e.set_tar(pr.tar)
        q = dic.grid_queue(416, 384, radius, 5)
        e.process_pair(q)
        assert e.tuning()[key]["tuned"] == 1, e.tuning()
    assert q.tobytes() == outs[0].tobytes()


def _to_oracle(O, q):
    pois = np.zeros(len(q), dtype=O.POI2D_DTYPE)
    pois["x"], pois["y"] = q["x"], q["y"]
    for name, idx in (("u", O.P_U), ("ux", O.P_UX), ("uy", O.P_UY), ("v", O.P_V), ("vx", O.P_VX), ("vy", O.P_VY)):
        pois["p"][:, idx] = q[name]
    for name, idx in (("u0", O.R_U0), ("v0", O.R_V0), ("zncc", O.R_ZNCC), ("iteration", O.R_ITER)):
        pois["r"][:, idx] = q[name]
    return pois


@pytest.mark.parametrize("pixels", [False, True])
@pytest.mark.parametrize("radius", [20, 31])
def test_pair_walk_matches_oracle_same_seed(dic, oracle_mod, radius, pixels):
    O = oracle_mod
    from fasticgn_gb300 import speckle
    pr = speckle.pair_affine(seed=radius, width=448, height=416)
    ref, tar = pr.ref.astype(np.float32), pr.tar.astype(np.float32)
    q = dic.grid_queue(448, 416, radius, 6)
    oq = _to_oracle(O, q)
    O.fftcc2d(ref, tar, oq, radius)
    g = q.copy()
    for f, idx in (("u", O.P_U), ("ux", O.P_UX), ("uy", O.P_UY), ("v", O.P_V), ("vx", O.P_VX), ("vy", O.P_VY)):
        g[f] = oq["p"][:, idx]
    g["zncc"] = oq["r"][:, O.R_ZNCC]
    from fasticgn_gb300 import _lib
    icgn = dic.ICGN2D1(radius, radius, 0.001, 10)
    icgn.engine.set_sampling(_lib.DIC_SAMPLE_PIXELS if pixels else _lib.DIC_SAMPLE_TABLE)
    icgn.setImages(pr.ref, pr.tar)
    icgn.compute(g)
    gx, gy = O.gradient(ref)
    O.icgn2d1(ref, gx, gy, O.bspline_prepare(tar), oq, radius)
    cpu = {"u": oq["p"][:, O.P_U], "v": oq["p"][:, O.P_V], "zncc": oq["r"][:, O.R_ZNCC]}
    res = C.compare_frame(cpu, {"u": g["u"], "v": g["v"], "zncc": g["zncc"]})
    assert res["pass"], res
    assert np.array_equal(C.failure_codes(cpu["zncc"]), C.failure_codes(g["zncc"]))
    assert np.mean(oq["r"][:, O.R_ITER] == g["iteration"]) >= 0.98
    both = (cpu["zncc"] >= 0) & (g["zncc"] >= 0)
    np.testing.assert_allclose(g["zncc"][both], cpu["zncc"][both], atol=1e-4)


@pytest.mark.parametrize("pixels", [False, True])
@pytest.mark.parametrize("radius", [16, 22])
def test_pair_walk_exact_self_match(dic, golden, radius, pixels):
    """Target = reference: s = 1, ZNSSD = 0 and dp = 0 bit for bit, so every subset clear of
    the constant blocks ends at zncc == 1 with u = v = 0 after one iteration; subsets inside a
    block end -5 as on the CPU."""
    g = golden("zero_texture")
    ref = g["ref"]
    h, w = ref.shape
    q = dic.grid_queue(w, h, radius, 2)
    with _engine(dic, radius, pixels) as e:
        for pw in (1, 2):
            if pixels:
                e.set_launch_shape(4, warps_per_cta=4, ctas_per_sm=0, warps_per_poi=pw, tile=pw % 2)
            else:
                e.set_launch_shape(2, warps_per_cta=4, ctas_per_sm=0, warps_per_poi=pw)
            e.set_ref(ref)
            e.set_tar(ref)
            qq = q.copy()
            e.process_pair(qq)
            rel = C.block_relation(qq["x"], qq["y"], radius, g["block_x"], int(g["block_y"]), int(g["block_side"]))
            outside = rel == 0
            assert outside.sum() > 50
            assert np.all(qq["zncc"][outside] == 1.0)
            assert np.all(qq["u"][outside] == 0.0) and np.all(qq["v"][outside] == 0.0)
            assert np.all(qq["iteration"][outside] == 1.0)


@pytest.mark.parametrize("radius", [18, 30])
def test_pair_walk_pixels_match_table(dic, radius):
    """Pixel and table sampling of the pair walk differ by float rounding only; flags agree."""
    from fasticgn_gb300 import speckle
    pr = speckle.pair_bumps(seed=300 + radius, width=448, height=400, max_disp=8.0, max_strain=0.02)
    outs = []
    for pixels in (True, False):
        with _engine(dic, radius, pixels) as e:
            e.set_ref(pr.ref)
            e.set_tar(pr.tar)
            q = dic.grid_queue(448, 400, radius, 6)
            e.process_pair(q)
        outs.append(q)
    px, tb = outs
    ok = (px["zncc"] >= 0) & (tb["zncc"] >= 0)
    assert ok.mean() > 0.9
    assert np.abs(px["u"] - tb["u"])[ok].max() <= 1e-3 and np.abs(px["v"] - tb["v"])[ok].max() <= 1e-3
    assert np.median(np.abs(px["u"] - tb["u"])[ok]) <= 1e-5
    assert (C.failure_codes(px["zncc"]) == C.failure_codes(tb["zncc"])).mean() >= 0.999


@pytest.mark.parametrize("width,dtype", [(418, np.uint16), (421, np.uint8), (403, np.float32)])
def test_pair_walk_pixels_odd_widths_and_types(dic, width, dtype):
    """Widths that are not a multiple of 4 (the padded-pitch plane under the TMA windows) and
    12-bit / float input: the pixel pair walk's staged and unstaged forms give the same bits,
    and match the table form to float rounding with identical flags."""
    from fasticgn_gb300 import speckle
    pr = speckle.pair_bumps(seed=700 + width, width=width, height=360, max_disp=6.0, max_strain=0.015)
    scale = {np.uint8: 1.0, np.uint16: 16.0, np.float32: 1.0}[dtype]
    ref = (pr.ref.astype(np.float32) * scale).astype(dtype)
    tar = (pr.tar.astype(np.float32) * scale).astype(dtype)
    radius = 22
    outs = {}
    for name, pixels, shape in (("tma", True, dict(warps_per_cta=2, warps_per_poi=2, tile=1)),
                                ("none", True, dict(warps_per_cta=4, warps_per_poi=1, tile=0)),
                                ("table", False, None)):
        with _engine(dic, radius, pixels) as e:
            if shape:
                e.set_launch_shape(4, ctas_per_sm=0, **shape)
            e.set_ref(ref)
            e.set_tar(tar)
            q = dic.grid_queue(width, 360, radius, 5)
            e.process_pair(q)
        outs[name] = q
    assert outs["tma"].tobytes() == outs["none"].tobytes()
    px, tb = outs["tma"], outs["table"]
    ok = (px["zncc"] >= 0) & (tb["zncc"] >= 0)
    assert ok.mean() > 0.9
    assert np.abs(px["u"] - tb["u"])[ok].max() <= 1e-3 and np.abs(px["v"] - tb["v"])[ok].max() <= 1e-3
    assert (C.failure_codes(px["zncc"]) == C.failure_codes(tb["zncc"])).mean() >= 0.999

"""GPU parity: the CUDA path through the C ABI against the CPU oracle and the reference's
golden cases.  Tolerances are the reference parity gate's (smoke/check_cpu_gpu_parity.py):
per frame median |du|,|dv| <= 1e-3 px, p99 <= 1e-2 px, max <= 0.5 px; FFTCC integer peaks
must be identical except where the two candidate peaks are equal to within 1e-5 of the
peak value in the oracle's own correlation map; validity flags must agree."""
import json

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


def from_oracle(O, pois, like):
    q = np.zeros(len(pois), dtype=like.dtype)
    q["x"], q["y"] = pois["x"], pois["y"]
    for name, idx in (("u", O.P_U), ("ux", O.P_UX), ("uy", O.P_UY), ("v", O.P_V), ("vx", O.P_VX), ("vy", O.P_VY)):
        q[name] = pois["p"][:, idx]
    for name, idx in (("u0", O.R_U0), ("v0", O.R_V0), ("zncc", O.R_ZNCC), ("iteration", O.R_ITER),
                      ("convergence", O.R_CONV)):
        q[name] = pois["r"][:, idx]
    return q


def fields(q):
    return {k: q[k] for k in q.dtype.names}


@pytest.fixture(scope="module")
def affine_pair():
    from fasticgn_gb300 import speckle
    return speckle.pair_affine()


# ----------------------------------------------------------------------------- planes

@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.float32])
def test_planes_bit_exact(dic, oracle_mod, dtype):
    """Gradient2D4 planes and the BicubicBspline table equal the CPU's bit for bit."""
    O = oracle_mod
    rng = np.random.default_rng(11)
    h, w = 97, 130
    if dtype == np.float32:
        ref = rng.uniform(0, 300, (h, w)).astype(np.float32)
        tar = rng.uniform(0, 300, (h, w)).astype(np.float32)
    else:
        top = 255 if dtype == np.uint8 else 4095
        ref = rng.integers(0, top + 1, (h, w)).astype(dtype)
        tar = rng.integers(0, top + 1, (h, w)).astype(dtype)
    with dic.Engine(7) as e:
        e.set_ref(ref)
        e.set_tar(tar)
        pack = e.read_plane(dic._lib.DIC_PLANE_REF_PACK, w, h)
        coef = e.read_plane(dic._lib.DIC_PLANE_TAR_COEF, w, h)
        tarf = e.read_plane(dic._lib.DIC_PLANE_TAR, w, h)
    gx, gy = O.gradient(ref.astype(np.float32))
    assert np.array_equal(pack[..., 0], ref.astype(np.float32))
    assert np.array_equal(pack[..., 1], gx)
    assert np.array_equal(pack[..., 2], gy)
    assert np.array_equal(tarf, tar.astype(np.float32))
    # device layout: plane k = coefficient row k of every texel; the CPU's is texel-major
    texel_major = coef.transpose(1, 2, 0, 3).reshape(h, w, 16)
    assert np.array_equal(texel_major, O.bspline_prepare(tar.astype(np.float32)))


# ----------------------------------------------------------------------------- FFTCC

def check_fftcc(O, ref, tar, radius, gq, oq):
    """Integer peaks equal except on (near-)exact ties in the oracle's correlation map."""
    ou, ov = oq["p"][:, O.P_U], oq["p"][:, O.P_V]
    mism = np.flatnonzero((gq["u"] != ou) | (gq["v"] != ov))
    m = 2 * radius
    for i in mism:
        # the map of the window at the initial guess, indexed by the peak offset u - u0
        u0, v0 = float(gq["u0"][i]), float(gq["v0"][i])
        cmap = O.fftcc2d_map(ref, tar, radius, float(gq["x"][i]), float(gq["y"][i]), u0, v0)
        assert cmap is not None, f"POI {i}: GPU computed a POI the oracle leaves untouched"
        def val(u, v):
            lu = int(round(float(u) - u0)) % m
            lv = int(round(float(v) - v0)) % m
            return cmap[lv, lu]
        peak = cmap.max()
        assert abs(val(gq["u"][i], gq["v"][i]) - val(ou[i], ov[i])) <= 1e-5 * abs(peak), \
            f"POI {i}: peak ({gq['u'][i]},{gq['v'][i]}) vs oracle ({ou[i]},{ov[i]})"
    assert len(mism) <= max(2, len(gq) // 1000)
    z_o = oq["r"][:, O.R_ZNCC]
    ok = np.isfinite(z_o)
    np.testing.assert_allclose(gq["zncc"][ok], z_o[ok], atol=2e-4)
    return len(mism)


def test_fftcc_matches_oracle_r15(dic, oracle_mod, affine_pair):
    O = oracle_mod
    ref, tar = affine_pair.ref, affine_pair.tar
    q = dic.grid_queue(512, 512, 15, 10)
    oq = to_oracle(O, q)
    f = dic.FFTCC2D(15, 15)
    f.setImages(ref, tar)
    f.compute(q)
    O.fftcc2d(ref.astype(np.float32), tar.astype(np.float32), oq, 15)
    check_fftcc(O, ref.astype(np.float32), tar.astype(np.float32), 15, q, oq)
    # an integer peak lies within a pixel of the truth
    ut, vt = affine_pair.field(q["x"].astype(np.float64), q["y"].astype(np.float64))
    assert np.median(np.abs(q["u"] - ut)) < 1.0 and np.median(np.abs(q["v"] - vt)) < 1.0


@pytest.mark.parametrize("radius", [3, 4, 5, 6, 7, 9, 10, 11, 12, 13, 14, 16, 17, 18, 20, 21, 22, 24, 25, 26, 27, 28, 30, 31, 32])
def test_fftcc_matches_oracle_radii(dic, oracle_mod, radius):
    """Register FFT (2r <= 32) and the large-radius path against the oracle, shifted speckle.
    Every prime-factor split of k_fftcc2 is covered: 2r = 6, 10, 14, 18, 22, 26 (2 x odd),
    12, 20, 28 (4 x odd), 24 (8 x 3), 30 (2 x 3 x 5, the headline test); 8 and 16 are powers
    of two (Cooley-Tukey)."""
    O = oracle_mod
    from fasticgn_gb300 import speckle
    pr = speckle.pair_affine(seed=radius, width=256, height=224)
    ref, tar = pr.ref.astype(np.float32), pr.tar.astype(np.float32)
    q = dic.grid_queue(256, 224, radius, 7)
    q["u"] = -3.0                     # exercises the initial-guess offset of the target window
    q["v"] = 1.0
    oq = to_oracle(O, q)
    f = dic.FFTCC2D(radius, radius)
    f.setImages(pr.ref, pr.tar)
    f.compute(q)
    O.fftcc2d(ref, tar, oq, radius)
    check_fftcc(O, ref, tar, radius, q, oq)


def test_fftcc_out_of_bounds_untouched(dic):
    rng = np.random.default_rng(1)
    ref = rng.integers(0, 255, (64, 64)).astype(np.uint8)
    q = dic.make_queue([5.0, 32.0, 60.0], [32.0, 32.0, 32.0])
    q["u"][1] = 40.0                      # target window leaves the image
    q["zncc"] = 0.25
    before = q.copy()
    f = dic.FFTCC2D(8, 8)
    f.setImages(ref, ref)
    f.compute(q)
    assert q.tobytes() == before.tobytes()


def test_fftcc_indexed_validation(dic):
    """FFTCC2D::compute(queue, cache_indices) errors (src/oc_fftcc.cpp:498-527)."""
    rng = np.random.default_rng(2)
    ref = rng.integers(0, 255, (96, 96)).astype(np.uint8)
    f = dic.FFTCC2D(10, 10)
    f.setImages(ref, ref)
    q = dic.grid_queue(96, 96, 10, 20)
    with pytest.raises(RuntimeError):
        f.compute(q.copy(), np.arange(len(q)))        # no prepared layout yet
    f.prepareRef(q)
    with pytest.raises(IndexError):
        f.compute(q.copy(), np.full(len(q), len(q)))
    with pytest.raises(ValueError):
        f.compute(q.copy(), np.roll(np.arange(len(q)), 1))
    with pytest.raises(ValueError):
        f.compute(q.copy(), np.arange(len(q) - 1))
    out = f.compute(q.copy(), np.arange(len(q)))
    plain = f.compute(q.copy())
    assert out.tobytes() == plain.tobytes()
    with pytest.raises(ValueError):
        dic.FFTCC2D(10, 12)


# ----------------------------------------------------------------------------- IC-GN

def test_icgn_matches_oracle_same_seed(dic, oracle_mod, affine_pair):
    """Identical FFTCC seeds in, IC-GN out: displacement parity and identical flags."""
    O = oracle_mod
    ref, tar = affine_pair.ref.astype(np.float32), affine_pair.tar.astype(np.float32)
    q = dic.grid_queue(512, 512, 15, 5)
    oq = to_oracle(O, q)
    O.fftcc2d(ref, tar, oq, 15)
    seeded = from_oracle(O, oq, q)
    g = seeded.copy()
    icgn = dic.ICGN2D1(15, 15, 0.001, 10)
    icgn.setImages(affine_pair.ref, affine_pair.tar)
    icgn.compute(g)
    gx, gy = O.gradient(ref)
    O.icgn2d1(ref, gx, gy, O.bspline_prepare(tar), oq, 15)
    cpu = from_oracle(O, oq, q)
    res = C.compare_frame(fields(cpu), fields(g))
    assert res["pass"], res
    neg_cpu = np.where(cpu["zncc"] < 0, cpu["zncc"], 0)
    neg_gpu = np.where(g["zncc"] < 0, g["zncc"], 0)
    assert np.mean(neg_cpu == neg_gpu) >= 0.999
    assert np.mean(cpu["iteration"] == g["iteration"]) >= 0.98
    both = (cpu["zncc"] >= 0) & (g["zncc"] >= 0)
    np.testing.assert_allclose(g["zncc"][both], cpu["zncc"][both], atol=1e-4)
    for k in ("ux", "uy", "vx", "vy"):
        assert np.median(np.abs(g[k][both] - cpu[k][both])) <= 1e-5


def test_pair_parity_config1(dic, oracle_mod, affine_pair):
    """512x512 pair, r=15, step 10: FFTCC seed + IC-GN, engine vs oracle run_pair."""
    O = oracle_mod
    q = dic.grid_queue(512, 512, 15, 10)
    oq = to_oracle(O, q)
    e = dic.Engine(15)
    e.set_ref(affine_pair.ref)
    e.set_tar(affine_pair.tar)
    e.process_pair(q)
    O.run_pair(affine_pair.ref.astype(np.float32), affine_pair.tar.astype(np.float32), oq, 15)
    res = C.compare_frame(fields(from_oracle(O, oq, q)), fields(q))
    assert res["pass"], res
    C.assert_flags_agree(fields(from_oracle(O, oq, q)), fields(q))
    ut, vt = affine_pair.field(q["x"].astype(np.float64), q["y"].astype(np.float64))
    ok = q["zncc"] >= 0
    assert np.sqrt(np.mean((q["u"][ok] - ut[ok]) ** 2)) < 0.02


@pytest.mark.parametrize("case", ["s15", "s15_lowsnr", "s63"])
def test_golden_accuracy_and_parity(dic, oracle_mod, golden, case):
    """The reference's sub-pixel accuracy gate cases: limits vs truth, parity vs the oracle."""
    O = oracle_mod
    g = golden(case)
    limits = json.loads(str(g["limits"]))
    ref, radius, grid = g["ref"], int(g["radius"]), int(g["grid"])
    h, w = ref.shape
    e = dic.Engine(radius)
    e.set_ref(ref)
    for k, motion in enumerate(g["motions"]):
        tar = g["tars"][k]
        q = dic.grid_queue(w, h, radius, grid)
        oq = to_oracle(O, q)
        e.set_tar(tar)
        e.process_pair(q)
        m = C.accuracy(fields(q), motion, g["centre"], w, h, radius)
        assert not C.check_accuracy(m, limits), (case, k, m)
        O.run_pair(ref.astype(np.float32), tar.astype(np.float32), oq, radius)
        res = C.compare_frame(fields(from_oracle(O, oq, q)), fields(q), min_shared_valid=50)
        assert res["pass"], (case, k, res)
        C.assert_flags_agree(fields(from_oracle(O, oq, q)), fields(q))


def test_whole_pixel_shifts_exact(dic, golden):
    g = golden("shift")
    ref, radius = g["ref"], int(g["radius"])
    h, w = ref.shape
    e = dic.Engine(radius)
    e.set_ref(ref)
    for (dx, dy), tar in zip(g["shifts"], g["tars"]):
        q = dic.grid_queue(w, h, radius, 1)
        e.set_tar(tar)
        e.process_pair(q)
        x, y = q["x"], q["y"]
        inside = (x - radius - 2 >= dx + 1) & (y - radius - 2 >= dy + 1) & \
                 (x + dx + radius + 3 < w) & (y + dy + radius + 3 < h)
        assert inside.sum() > 100
        assert np.all(np.abs(q["u"][inside] - dx) <= 1e-4)
        assert np.all(np.abs(q["v"][inside] - dy) <= 1e-4)
        assert np.all(q["zncc"][inside] >= 0.9999)


def test_oob_band(dic, golden):
    g = golden("oob")
    ref, tar, radius, shift = g["ref"], g["tar"], int(g["radius"]), int(g["shift"])
    h, w = ref.shape
    q = dic.grid_queue(w, h, radius, 1)
    q["u"] = shift
    icgn = dic.ICGN2D1(radius, radius, 0.001, 10)
    icgn.setImages(ref, tar)
    icgn.compute(q)
    band = C.oob_band(q["x"], q["y"], radius, w, h, shift, 0)
    assert band.sum() > 0
    assert np.all(q["zncc"][band] == -3.0)
    assert np.all(q["u"][band] == shift)
    assert np.all(q["zncc"][~band] != -3.0)


def test_zero_texture_cpu_rule(dic, golden):
    """Same outcome as the CPU backend: -5 and u = v = 0 inside a constant block; an exact
    self-match (zncc == 1, |u|,|v| <= 1e-4) outside every block."""
    g = golden("zero_texture")
    ref, radius = g["ref"], int(g["radius"])
    h, w = ref.shape
    q = dic.grid_queue(w, h, radius, 1)
    e = dic.Engine(radius)
    e.set_ref(ref)
    e.set_tar(ref)
    e.process_pair(q)
    rel = C.block_relation(q["x"], q["y"], radius, g["block_x"], int(g["block_y"]), int(g["block_side"]))
    inside, outside = rel == 2, rel == 0
    assert inside.sum() > 0
    assert np.all(q["zncc"][inside] == -5.0)
    assert np.all(q["u"][inside] == 0.0) and np.all(q["v"][inside] == 0.0)
    assert np.all(q["zncc"][outside] == 1.0)
    assert np.all(np.abs(q["u"][outside]) <= 1e-4) and np.all(np.abs(q["v"][outside]) <= 1e-4)
    # shifted target with the blocks repainted: zero-texture POIs still -5 with u = v = 0
    q2 = dic.grid_queue(w, h, radius, 1)
    e.set_tar(g["tar_shift"])
    e.process_pair(q2)
    assert np.all(q2["zncc"][inside] == -5.0)


def test_entry_test_rules(dic, oracle_mod):
    """src/oc_icgn.cpp:184-191: a negative incoming zncc is kept, a seed beyond the image or a
    subset past the border gives -3, NaN seeds give -3; nothing else changes."""
    O = oracle_mod
    rng = np.random.default_rng(4)
    ref = rng.integers(0, 255, (80, 80)).astype(np.uint8)
    q = dic.make_queue([40, 40, 40, 3, 40, 40], [40, 40, 40, 40, 40, 40])
    q["zncc"] = [-0.5, 0.3, 0.3, 0.3, np.nan, 0.3]
    q["u"] = [0, 80.0, 0, 0, 0, np.nan]
    q["iteration"] = 7
    oq = to_oracle(O, q)
    icgn = dic.ICGN2D1(5, 5, 0.001, 10)
    icgn.setImages(ref, ref)
    icgn.compute(q)
    gx, gy = O.gradient(ref.astype(np.float32))
    O.icgn2d1(ref.astype(np.float32), gx, gy, O.bspline_prepare(ref.astype(np.float32)), oq, 5)
    cpu = from_oracle(O, oq, q)
    assert q["zncc"][0] == -0.5 and q["zncc"][1] == -3.0 and q["zncc"][3] == -3.0
    assert q["zncc"][5] == -3.0
    for i in (0, 1, 3, 5):
        assert q[i].tobytes() == cpu[i].tobytes()
    # NaN < 0 is false, so a NaN incoming zncc is solved like any other POI (here a self-match)
    for i in (2, 4):
        assert q["iteration"][i] >= 1 and q["zncc"][i] == 1.0 and cpu["zncc"][i] == 1.0


def test_deterministic_and_device_path(dic, affine_pair):
    """Byte-identical reruns; the device-resident entry point equals the host one."""
    torch = pytest.importorskip("torch")
    q1 = dic.grid_queue(512, 512, 15, 6)
    q2 = q1.copy()
    e = dic.Engine(15)
    e.set_ref(affine_pair.ref)
    e.set_tar(affine_pair.tar)
    e.process_pair(q1)
    e.process_pair(q2)
    assert q1.tobytes() == q2.tobytes()
    q3 = dic.grid_queue(512, 512, 15, 6)
    dev = torch.from_numpy(q3.view(np.uint8).copy()).cuda()
    e2 = dic.Engine(15)
    ref_d = torch.from_numpy(affine_pair.ref).cuda()
    tar_d = torch.from_numpy(affine_pair.tar).cuda()
    torch.cuda.synchronize()
    e2.set_ref_device(ref_d.data_ptr(), 512, 512, 512, dic._lib.DIC_U8)
    e2.set_tar_device(tar_d.data_ptr(), 512, 512, 512, dic._lib.DIC_U8)
    e2.run_device(dev.data_ptr(), len(q3), dic._lib.DIC_RUN_FFTCC | dic._lib.DIC_RUN_ICGN)
    st = e2.stats()
    out = dev.cpu().numpy().view(dic.POI_DTYPE)
    assert out.tobytes() == q1.tobytes()
    assert st["kernel_launches"] >= 5 and st["icgn_iterations"] > len(q1)


def test_u16_12bit_and_scale(dic, oracle_mod):
    """12-bit data in uint16 (right aligned) and left-aligned data read with scale 1/16."""
    O = oracle_mod
    from fasticgn_gb300 import speckle
    ref, frames = speckle.stream_frames(width=256, height=256, frames=4, which=[3])
    _, tar, field = frames[0]
    q = dic.grid_queue(256, 256, 12, 8)
    oq = to_oracle(O, q)
    e = dic.Engine(12)
    e.set_ref(ref)
    e.set_tar(tar)
    e.process_pair(q)
    O.run_pair(ref.astype(np.float32), tar.astype(np.float32), oq, 12)
    res = C.compare_frame(fields(from_oracle(O, oq, q)), fields(q))
    assert res["pass"], res
    C.assert_flags_agree(fields(from_oracle(O, oq, q)), fields(q))
    q2 = dic.grid_queue(256, 256, 12, 8)
    e2 = dic.Engine(12, input_scale=1.0 / 16.0)
    e2.set_ref((ref.astype(np.uint32) << 4).astype(np.uint16))
    e2.set_tar((tar.astype(np.uint32) << 4).astype(np.uint16))
    e2.process_pair(q2)
    assert q2.tobytes() == q.tobytes()


def test_state_errors(dic):
    e = dic.Engine(7)
    q = dic.grid_queue(64, 64, 7, 8)
    with pytest.raises(RuntimeError):
        e.icgn(q)
    e.set_ref(np.zeros((64, 64), np.uint8))
    with pytest.raises(ValueError):
        e.set_tar(np.zeros((64, 65), np.uint8))
    with pytest.raises(ValueError):
        e.set_ref(np.zeros((64, 64, 3), np.uint8))


def test_oversize_image_rejected(dic):
    """Texel indices are 32-bit: an image of 2^31 pixels or more is refused before any byte
    of it is read (the declared size is what is checked; the buffer here is one row)."""
    from fasticgn_gb300 import _lib
    e = dic.Engine(7)
    row = np.zeros(65536, np.uint8)
    L = _lib.load()
    rc = L.dic_set_ref(e._h, row.ctypes.data, 65536, 32768, 65536, _lib.DIC_U8)
    assert rc == _lib.DIC_ERR_ARGUMENT
    assert b"2^31" in L.dic_last_error(e._h)
    e.set_ref(np.zeros((64, 64), np.uint8))   # the engine is still usable
    e.close()


@pytest.mark.parametrize("case", ["u8_dark", "u16_bright"])
def test_illumination_change_pair(dic, oracle_mod, case):
    """Target = a * I + b (a brightness and contrast change, which ZNCC / ZNSSD is invariant
    to): 0.6 I - 20 DN on 8-bit data and 1.4 I + 600 DN on 12-bit data.  The IC-GN kernels form
    the zero-mean sums from offsets to the reference mean in one pass; against the oracle's
    two-pass Eigen arithmetic the results stay within the parity gate with identical flags,
    and the displacements still match the truth."""
    O = oracle_mod
    from fasticgn_gb300 import speckle
    if case == "u8_dark":
        pr = speckle.pair_affine(seed=7, width=512, height=512)
        ref = pr.ref
        tar = np.clip(np.rint(0.6 * pr.tar.astype(np.float64) - 20.0), 0, 255).astype(np.uint8)
        assert pr.tar.min() >= 34      # no clipping: the change is exactly affine before rounding
        field, radius, step = pr.field, 15, 7
    else:
        ref, frames = speckle.stream_frames(width=512, height=512, frames=200, which=[150])
        _, t12, field = frames[0]
        tar = np.rint(1.4 * t12.astype(np.float64) + 600.0).astype(np.uint16)
        radius, step = 15, 7
    h, w = ref.shape
    q = dic.grid_queue(w, h, radius, step)
    oq = to_oracle(O, q)
    e = dic.Engine(radius)
    e.set_ref(ref)
    e.set_tar(tar)
    e.process_pair(q)
    e.close()
    O.run_pair(ref.astype(np.float32), tar.astype(np.float32), oq, radius)
    cpu = fields(from_oracle(O, oq, q))
    res = C.compare_frame(cpu, fields(q))
    assert res["pass"], (case, res)
    C.assert_flags_agree(cpu, fields(q))
    ok = q["zncc"] >= 0
    assert ok.mean() > 0.95
    np.testing.assert_allclose(q["zncc"][ok & (cpu["zncc"] >= 0)], cpu["zncc"][ok & (cpu["zncc"] >= 0)], atol=1e-4)
    ut, vt = field(q["x"].astype(np.float64), q["y"].astype(np.float64))
    assert np.sqrt(np.mean((q["u"][ok] - ut[ok]) ** 2)) < 0.03
    assert np.sqrt(np.mean((q["v"][ok] - vt[ok]) ** 2)) < 0.03

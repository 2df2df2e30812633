"""Seeded synthetic speckle pairs with exact displacement truth.

Images are sums of Gaussian speckles rendered analytically: the target pixel x' is mapped
back to its material point X (x' = X + d(X), solved by fixed-point iteration, which
converges because the displacement gradients stay far below 1) and the reference pattern
is evaluated at X.  No image is resampled, so the truth d(X) at every reference POI is
exact and a first-order subset shape function sees no model error for affine fields.

Workload shapes (all sizes in px, values in grey levels):

* ``pair_affine``: 512x512 u8, background 40, ~3000 speckles with sigma ~ U(1.5, 3) and
  peak ~ U(80, 200), translation (2.37, -1.61) plus uniform strain 1e-3, noise 1 DN.
* ``pair_bumps``: 2048x2048 u8, the same speckle density, displacement = sum of 8 Gaussian
  bumps scaled to |u|, |v| <= 12 px and local strain <= 2 %, noise 2 DN.
* ``stream_frame``: 2048x2048 12-bit in u16, affine strain ramp + a sinusoidal
  displacement of wavelength 256 px, noise 8 DN.
* ``crack_frames``: 1024x1024 12-bit in u16, uniform strain ramping to 3e-3 + a displacement
  jump across a random line growing to 1.5 px, noise 6 DN.
* ``uneven_batch``: pairs with sides log-uniform in 256..4096 u8, each with its own random
  affine field (|u|, |v| <= 8 px, strains <= 1 %), 20 % of the area replaced by flat
  low-texture patches, subset radius drawn from {10, 15, 20, 30} and a POI count
  log-uniform in 1k..600k (as far as the image holds).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

SPECKLES_PER_PX = 3000.0 / (512.0 * 512.0)


@dataclasses.dataclass
class Speckles:
    x: np.ndarray
    y: np.ndarray
    sigma: np.ndarray
    peak: np.ndarray


def make_speckles(rng: np.random.Generator, width: int, height: int, pad: float,
                  density: float = SPECKLES_PER_PX, sigma=(1.5, 3.0), peak=(80.0, 200.0)) -> Speckles:
    area = (width + 2 * pad) * (height + 2 * pad)
    n = int(round(density * area))
    return Speckles(x=rng.uniform(-pad, width + pad, n), y=rng.uniform(-pad, height + pad, n),
                    sigma=rng.uniform(sigma[0], sigma[1], n), peak=rng.uniform(peak[0], peak[1], n))


def render(width: int, height: int, sp: Speckles, field=None, background: float = 40.0,
           chunk: int = 2048) -> np.ndarray:
    """Float64 image of the speckle pattern carried by ``field`` (None = reference).

    ``field(X, Y) -> (u, v)`` is the displacement of the material point at reference (X, Y).
    """
    yy, xx = np.meshgrid(np.arange(height, dtype=np.float64), np.arange(width, dtype=np.float64),
                         indexing="ij")
    if field is None:
        bx, by = xx, yy
        fx, fy = sp.x, sp.y
    else:
        bx, by = xx.copy(), yy.copy()
        # X = x' - d(X); the error contracts by max|grad d| <= 0.02 per pass, so six passes
        # leave < 1e-8 px for a 12 px field.
        for _ in range(6):
            u, v = field(bx, by)
            bx, by = xx - u, yy - v
        su, sv = field(sp.x, sp.y)
        fx, fy = sp.x + su, sp.y + sv
    img = np.full(width * height, background, dtype=np.float64)
    reach = int(math.ceil(4.0 * float(sp.sigma.max()) + 2.0))
    off = np.arange(-reach, reach + 1)
    oy, ox = np.meshgrid(off, off, indexing="ij")
    oy, ox = oy.ravel(), ox.ravel()
    bxf, byf = bx.ravel(), by.ravel()
    for s in range(0, len(sp.x), chunk):
        cx = np.rint(fx[s:s + chunk]).astype(np.int64)
        cy = np.rint(fy[s:s + chunk]).astype(np.int64)
        px = cx[:, None] + ox[None, :]
        py = cy[:, None] + oy[None, :]
        inside = (px >= 0) & (px < width) & (py >= 0) & (py < height)
        idx = np.where(inside, py * width + px, 0)
        dx = bxf[idx] - sp.x[s:s + chunk, None]
        dy = byf[idx] - sp.y[s:s + chunk, None]
        sig = sp.sigma[s:s + chunk, None]
        val = sp.peak[s:s + chunk, None] * np.exp(-(dx * dx + dy * dy) / (2.0 * sig * sig))
        val = np.where(inside, val, 0.0)
        img += np.bincount(idx.ravel(), weights=val.ravel(), minlength=width * height)
    return img.reshape(height, width)


def quantize(img: np.ndarray, rng: np.random.Generator, noise: float, max_value: int,
             dtype) -> np.ndarray:
    out = img + (rng.normal(0.0, noise, img.shape) if noise > 0 else 0.0)
    return np.clip(np.rint(out), 0, max_value).astype(dtype)


# --------------------------------------------------------------------------- fields

def affine_field(u0, v0, ux, uy, vx, vy, xc, yc):
    def f(x, y):
        return (u0 + ux * (x - xc) + uy * (y - yc), v0 + vx * (x - xc) + vy * (y - yc))
    f.params = (u0, v0, ux, uy, vx, vy, xc, yc)
    return f


def bumps_field(rng: np.random.Generator, width: int, height: int, n: int = 8,
                max_disp: float = 12.0, max_strain: float = 0.02):
    """Sum of n Gaussian bumps per component, scaled to the displacement/strain limits."""
    cx = rng.uniform(0, width, (2, n))
    cy = rng.uniform(0, height, (2, n))
    s = rng.uniform(0.15, 0.35, (2, n)) * max(width, height)
    a = rng.uniform(-1.0, 1.0, (2, n))

    def raw(x, y, k):
        out = np.zeros(np.broadcast(x, y).shape)
        for j in range(n):
            out = out + a[k, j] * np.exp(-((x - cx[k, j]) ** 2 + (y - cy[k, j]) ** 2) / (2 * s[k, j] ** 2))
        return out

    gy, gx = np.meshgrid(np.linspace(0, height - 1, 257), np.linspace(0, width - 1, 257), indexing="ij")
    scale = 1.0
    for k in range(2):
        f = raw(gx, gy, k)
        du_dy, du_dx = np.gradient(f, gy[:, 0], gx[0, :])
        disp = np.abs(f).max()
        strain = max(np.abs(du_dx).max(), np.abs(du_dy).max())
        scale = min(scale, max_disp / disp, max_strain / strain)

    def field(x, y):
        return scale * raw(x, y, 0), scale * raw(x, y, 1)
    return field


def sine_field(amp: float, wavelength: float, strain: float, xc: float, yc: float):
    def field(x, y):
        return (strain * (x - xc) + amp * np.sin(2 * np.pi * x / wavelength),
                strain * (y - yc) + amp * np.sin(2 * np.pi * y / wavelength))
    return field


def crack_field(strain: float, jump: float, p0, direction, xc: float, yc: float):
    nx, ny = -direction[1], direction[0]

    def field(x, y):
        side = ((x - p0[0]) * nx + (y - p0[1]) * ny) > 0
        return (strain * (x - xc) + np.where(side, jump * nx, 0.0),
                strain * (y - yc) + np.where(side, jump * ny, 0.0))
    return field


# --------------------------------------------------------------------------- workloads

@dataclasses.dataclass
class Pair:
    ref: np.ndarray          # raw pixels (u8 or u16)
    tar: np.ndarray
    field: object            # truth: field(x, y) -> (u, v) at reference positions
    max_value: int


def pair_affine(seed: int = 1, width: int = 512, height: int = 512, noise: float = 1.0) -> Pair:
    rng = np.random.default_rng(seed)
    xc, yc = (width - 1) / 2.0, (height - 1) / 2.0
    field = affine_field(2.37, -1.61, 1e-3, 0.0, 0.0, 1e-3, xc, yc)
    sp = make_speckles(rng, width, height, pad=16.0)
    ref = quantize(render(width, height, sp), rng, noise, 255, np.uint8)
    tar = quantize(render(width, height, sp, field), rng, noise, 255, np.uint8)
    return Pair(ref, tar, field, 255)


def pair_bumps(seed: int = 4, width: int = 2048, height: int = 2048, noise: float = 2.0,
               max_disp: float = 12.0, max_strain: float = 0.02) -> Pair:
    rng = np.random.default_rng(seed)
    field = bumps_field(rng, width, height, max_disp=max_disp, max_strain=max_strain)
    sp = make_speckles(rng, width, height, pad=max_disp + 16.0)
    ref = quantize(render(width, height, sp), rng, noise, 255, np.uint8)
    tar = quantize(render(width, height, sp, field), rng, noise, 255, np.uint8)
    return Pair(ref, tar, field, 255)


def flat_patches(rng: np.random.Generator, width: int, height: int, fraction: float = 0.2):
    """Boolean mask of random rectangles covering about ``fraction`` of the image."""
    mask = np.zeros((height, width), dtype=bool)
    target = fraction * width * height
    while mask.sum() < target:
        pw = int(rng.uniform(0.05, 0.25) * width) + 8
        ph = int(rng.uniform(0.05, 0.25) * height) + 8
        x0 = int(rng.integers(0, max(1, width - pw)))
        y0 = int(rng.integers(0, max(1, height - ph)))
        mask[y0:y0 + ph, x0:x0 + pw] = True
    return mask


@dataclasses.dataclass
class BatchPair:
    ref: np.ndarray
    tar: np.ndarray
    field: object
    radius: int
    step: int
    flat: np.ndarray         # True inside the flat patches


def pair_uneven(rng: np.random.Generator, width: int, height: int, radius: int, pois: int,
                noise: float = 1.0, flat_fraction: float = 0.2) -> BatchPair:
    """One pair of the uneven batch: random affine field, flat patches (background plus
    noise only, in both images) and a POI step giving about ``pois`` grid POIs."""
    xc, yc = (width - 1) / 2.0, (height - 1) / 2.0
    u0, v0 = rng.uniform(-8.0, 8.0, 2)
    grads = rng.uniform(-0.01, 0.01, 4)
    half = max(width, height) / 2.0
    # keep |u|, |v| <= 8 px over the image: shrink the translation where the strain adds up
    lim_u = 8.0 - (abs(grads[0]) + abs(grads[1])) * half
    lim_v = 8.0 - (abs(grads[2]) + abs(grads[3])) * half
    if lim_u < 0 or lim_v < 0:
        grads = grads * min(1.0, 6.0 / ((np.abs(grads).max() * 2.0) * half))
        lim_u = 8.0 - (abs(grads[0]) + abs(grads[1])) * half
        lim_v = 8.0 - (abs(grads[2]) + abs(grads[3])) * half
    u0 = float(np.clip(u0, -lim_u, lim_u))
    v0 = float(np.clip(v0, -lim_v, lim_v))
    field = affine_field(u0, v0, *grads, xc, yc)
    sp = make_speckles(rng, width, height, pad=24.0)
    ref_f = render(width, height, sp)
    tar_f = render(width, height, sp, field)
    flat = flat_patches(rng, width, height, flat_fraction)
    ref_f[flat] = 40.0
    tar_f[flat] = 40.0
    ref = quantize(ref_f, rng, noise, 255, np.uint8)
    tar = quantize(tar_f, rng, noise, 255, np.uint8)
    margin = radius + 2
    span = max(1, min(width, height) - 2 * margin)
    step = max(1, int(math.ceil(math.sqrt((width - 2 * margin) * (height - 2 * margin) / float(pois)))))
    step = min(step, span)
    return BatchPair(ref, tar, field, radius, step, flat)


def uneven_specs(seed: int = 3, count: int = 16, min_side: int = 256, max_side: int = 4096,
                 radii=(10, 15, 20, 30), min_pois: int = 1000, max_pois: int = 600_000):
    """Shapes of the uneven batch: (pair seed, width, height, radius, POI count) per pair."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        w = int(round(math.exp(rng.uniform(math.log(min_side), math.log(max_side)))))
        h = int(round(math.exp(rng.uniform(math.log(min_side), math.log(max_side)))))
        r = int(rng.choice(radii))
        n = int(round(math.exp(rng.uniform(math.log(min_pois), math.log(max_pois)))))
        out.append((seed * 1000 + k, w, h, r, n))
    return out


def render_uneven(spec) -> BatchPair:
    seed, w, h, r, n = spec
    return pair_uneven(np.random.default_rng(seed), w, h, r, n)


def render_uneven_job(spec):
    """(ref, tar, radius, step) of one uneven-batch pair (picklable, for worker pools)."""
    p = render_uneven(spec)
    return p.ref, p.tar, p.radius, p.step


def uneven_batch(seed: int = 3, count: int = 16, **kw):
    """The uneven batch: ``count`` pairs of random size, radius and POI count."""
    return [render_uneven(s) for s in uneven_specs(seed, count, **kw)]


def stream_frames(seed: int = 2, width: int = 2048, height: int = 2048, frames: int = 200,
                  which=None, noise: float = 8.0):
    """Reference + the requested frames of the 12-bit sine/strain stream (frame k of `frames`)."""
    rng = np.random.default_rng(seed)
    sp = make_speckles(rng, width, height, pad=24.0, peak=(80.0 * 4095 / 255, 200.0 * 4095 / 255))
    bg = 40.0 * 4095 / 255
    ref = quantize(render(width, height, sp, background=bg), rng, noise, 4095, np.uint16)
    out = []
    xc, yc = (width - 1) / 2.0, (height - 1) / 2.0
    for k in (which if which is not None else range(frames)):
        frac = (k + 1) / frames
        field = sine_field(0.5 * frac, 256.0, 5e-3 * frac, xc, yc)
        frng = np.random.default_rng(seed * 100003 + k)
        tar = quantize(render(width, height, sp, field, background=bg), frng, noise, 4095, np.uint16)
        out.append((k, tar, field))
    return ref, out


def crack_setup(seed: int = 5, width: int = 1024, height: int = 1024):
    """Reference and crack geometry of the high-speed crack stream: a random line through
    the middle half of the image, 12-bit speckle (values scaled to 4095)."""
    rng = np.random.default_rng(seed)
    sp = make_speckles(rng, width, height, pad=24.0, peak=(80.0 * 4095 / 255, 200.0 * 4095 / 255))
    p0 = (rng.uniform(0.35, 0.65) * width, rng.uniform(0.35, 0.65) * height)
    ang = rng.uniform(0.0, np.pi)
    direction = (float(np.cos(ang)), float(np.sin(ang)))
    return rng, sp, p0, direction


def crack_frames(seed: int = 5, width: int = 1024, height: int = 1024, frames: int = 5000, which=None,
                 noise: float = 6.0, max_strain: float = 3e-3, max_jump: float = 1.5):
    """Reference + requested frames of the crack stream: uniform strain ramping to
    ``max_strain`` plus a displacement jump across the crack line growing to ``max_jump`` px
    (normal to the line), noise ``noise`` DN, 12-bit values in u16.  Returns
    (ref, [(k, tar, field)], crack) with crack = (p0, direction)."""
    rng, sp, p0, direction = crack_setup(seed, width, height)
    bg = 40.0 * 4095 / 255
    ref = quantize(render(width, height, sp, background=bg), rng, noise, 4095, np.uint16)
    xc, yc = (width - 1) / 2.0, (height - 1) / 2.0
    out = []
    for k in (which if which is not None else range(frames)):
        frac = (k + 1) / frames
        field = crack_field(max_strain * frac, max_jump * frac, p0, direction, xc, yc)
        frng = np.random.default_rng(seed * 100003 + k)
        tar = quantize(render(width, height, sp, field, background=bg), frng, noise, 4095, np.uint16)
        out.append((k, tar, field))
    return ref, out, (p0, direction)


def crack_distance(x, y, crack):
    """Distance of (x, y) from the crack line."""
    (px, py), (dx, dy) = crack
    return np.abs((np.asarray(x) - px) * (-dy) + (np.asarray(y) - py) * dx)


def stream_image(spec):
    """One image of a stream, picklable for worker pools: spec = (kind, seed, width, height,
    frames, k) with kind "stream" (stream_frames) or "crack" (crack_frames) and k = -1 for
    the reference.  Gives the same pixels as those functions."""
    kind, seed, width, height, frames, k = spec
    bg = 40.0 * 4095 / 255
    if kind == "stream":
        rng = np.random.default_rng(seed)
        sp = make_speckles(rng, width, height, pad=24.0, peak=(80.0 * 4095 / 255, 200.0 * 4095 / 255))
        noise = 8.0
        xc, yc = (width - 1) / 2.0, (height - 1) / 2.0
        frac = (k + 1) / frames
        field = sine_field(0.5 * frac, 256.0, 5e-3 * frac, xc, yc) if k >= 0 else None
    else:
        rng, sp, p0, direction = crack_setup(seed, width, height)
        noise = 6.0
        xc, yc = (width - 1) / 2.0, (height - 1) / 2.0
        frac = (k + 1) / frames
        field = crack_field(3e-3 * frac, 1.5 * frac, p0, direction, xc, yc) if k >= 0 else None
    if k < 0:
        return quantize(render(width, height, sp, background=bg), rng, noise, 4095, np.uint16)
    frng = np.random.default_rng(seed * 100003 + k)
    return quantize(render(width, height, sp, field, background=bg), frng, noise, 4095, np.uint16)


def grid_xy(width: int, height: int, radius: int, step: int):
    """POI grid of buildPoiQueue (opencorr_cli_cuda_mvp.cpp:2439-2472): margin r+2, y outer."""
    margin = radius + 2
    ys, xs = np.meshgrid(np.arange(margin, height - margin, step), np.arange(margin, width - margin, step),
                         indexing="ij")
    return xs.ravel().astype(np.float32), ys.ravel().astype(np.float32)

"""TEST INFRASTRUCTURE: ctypes view of oracle/libdic_oracle.so.

The oracle is a CPU restatement of OpenCorr's path (oc_gradient.cpp, oc_cubic_bspline.cpp,
oc_icgn.cpp, oc_fftcc.cpp); see dic_oracle.cpp for the line-by-line citations.  POIs are
numpy structured arrays with the memory layout of opencorr::POI2D (src/oc_poi.h:102-136).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB, build_oracle

POI2D_DTYPE = np.dtype([
    ("x", "<f4"), ("y", "<f4"),
    ("p", "<f4", (12,)),       # u ux uy uxx uxy uyy v vx vy vxx vxy vyy
    ("r", "<f4", (6,)),        # u0 v0 zncc iteration convergence feature
    ("e", "<f4", (3,)),
    ("subset_radius", "<f4", (2,)),
])
assert POI2D_DTYPE.itemsize == 100

P_U, P_UX, P_UY, P_V, P_VX, P_VY = 0, 1, 2, 6, 7, 8
R_U0, R_V0, R_ZNCC, R_ITER, R_CONV = 0, 1, 2, 3, 4

_lib = None


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle()
        L = ctypes.CDLL(str(path))
        f32p = ctypes.POINTER(ctypes.c_float)
        vp = ctypes.c_void_p
        L.oc_gradient.argtypes = [f32p, ctypes.c_int, ctypes.c_int, f32p, f32p, ctypes.c_int]
        L.oc_bspline_prepare.argtypes = [f32p, ctypes.c_int, ctypes.c_int, f32p, ctypes.c_int]
        L.oc_bspline_value.argtypes = [f32p, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float]
        L.oc_bspline_value.restype = ctypes.c_float
        L.oc_icgn2d1.argtypes = [f32p, f32p, f32p, f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_float, ctypes.c_float, vp, ctypes.c_longlong,
                                 ctypes.c_int]
        L.oc_fftcc2d.argtypes = [f32p, f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp,
                                 ctypes.c_longlong, ctypes.c_int]
        L.oc_fftcc2d_map.argtypes = [f32p, f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     f32p]
        L.oc_fftcc2d_map.restype = ctypes.c_int
        L.oc_run_pair.argtypes = [f32p, f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_float, ctypes.c_float, vp, ctypes.c_longlong, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_double)]
        _lib = L
    return _lib


def _f32(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def make_pois(xs, ys) -> np.ndarray:
    pois = np.zeros(len(xs), dtype=POI2D_DTYPE)
    pois["x"] = xs
    pois["y"] = ys
    return pois


def grid_pois(width: int, height: int, radius: int, step: int) -> np.ndarray:
    """buildPoiQueue (opencorr_cli_cuda_mvp.cpp:2439-2472): margin r+2, y outer, x inner."""
    margin = radius + 2
    ys, xs = np.meshgrid(np.arange(margin, height - margin, step, dtype=np.float32),
                         np.arange(margin, width - margin, step, dtype=np.float32), indexing="ij")
    return make_pois(xs.ravel(), ys.ravel())


def gradient(img: np.ndarray, threads: int | None = None):
    img = _f32(img)
    h, w = img.shape
    gx = np.empty_like(img)
    gy = np.empty_like(img)
    lib().oc_gradient(_ptr(img), w, h, _ptr(gx), _ptr(gy), threads or default_threads())
    return gx, gy


def bspline_prepare(img: np.ndarray, threads: int | None = None) -> np.ndarray:
    img = _f32(img)
    h, w = img.shape
    coef = np.empty((h, w, 16), dtype=np.float32)
    lib().oc_bspline_prepare(_ptr(img), w, h, _ptr(coef), threads or default_threads())
    return coef


def bspline_value(coef: np.ndarray, x: float, y: float) -> float:
    h, w = coef.shape[:2]
    return lib().oc_bspline_value(_ptr(coef), w, h, x, y)


def icgn2d1(ref, gx, gy, coef, pois: np.ndarray, radius: int, conv: float = 0.001,
            max_iter: int = 10, threads: int | None = None) -> np.ndarray:
    ref, gx, gy, coef = _f32(ref), _f32(gx), _f32(gy), _f32(coef)
    assert pois.dtype == POI2D_DTYPE and pois.flags.c_contiguous
    h, w = ref.shape
    lib().oc_icgn2d1(_ptr(ref), _ptr(gx), _ptr(gy), _ptr(coef), w, h, radius, radius, conv,
                     float(max_iter), pois.ctypes.data, len(pois), threads or default_threads())
    return pois


def fftcc2d(ref, tar, pois: np.ndarray, radius: int, threads: int | None = None) -> np.ndarray:
    ref, tar = _f32(ref), _f32(tar)
    assert pois.dtype == POI2D_DTYPE and pois.flags.c_contiguous
    h, w = ref.shape
    lib().oc_fftcc2d(_ptr(ref), _ptr(tar), w, h, radius, pois.ctypes.data, len(pois),
                     threads or default_threads())
    return pois


def fftcc2d_map(ref, tar, radius: int, x: float, y: float, u0: float = 0.0, v0: float = 0.0):
    ref, tar = _f32(ref), _f32(tar)
    h, w = ref.shape
    m = 2 * radius
    out = np.zeros((m, m), dtype=np.float32)
    ok = lib().oc_fftcc2d_map(_ptr(ref), _ptr(tar), w, h, radius, x, y, u0, v0, _ptr(out))
    return out if ok else None


def run_pair(ref, tar, pois: np.ndarray, radius: int, conv: float = 0.001, max_iter: int = 10,
             threads: int | None = None):
    """FFTCC seed then IC-GN1 on one pair; returns (pois, phase seconds[4])."""
    ref, tar = _f32(ref), _f32(tar)
    h, w = ref.shape
    t = (ctypes.c_double * 4)()
    lib().oc_run_pair(_ptr(ref), _ptr(tar), w, h, radius, conv, float(max_iter), pois.ctypes.data,
                      len(pois), threads or default_threads(), t)
    return pois, list(t)

"""ctypes binding of libdic.so (the C ABI declared in include/dic.h).

The library is required: there is no CPU fallback.  Importing the engine classes without
a built libdic.so raises at first use with the build command to run.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from ._build import LIB

DIC_OK = 0
DIC_ERR_ARGUMENT = -1
DIC_ERR_STATE = -2
DIC_ERR_RANGE = -3
DIC_ERR_CUDA = -4
DIC_ERR_MEMORY = -5

DIC_U8, DIC_U16, DIC_F32 = 1, 2, 3
DIC_RUN_FFTCC, DIC_RUN_ICGN, DIC_RUN_PREPARE, DIC_RUN_LEARNED = 1, 2, 4, 8
DIC_PIXELS_STAGED = 2
DIC_PLANE_REF, DIC_PLANE_REF_PACK, DIC_PLANE_TAR, DIC_PLANE_TAR_COEF = 1, 2, 3, 4
DIC_SAMPLE_TABLE, DIC_SAMPLE_PIXELS = 0, 1

# struct dic_poi (include/dic.h), 56 bytes
POI_DTYPE = np.dtype([
    ("x", "<f4"), ("y", "<f4"),
    ("u", "<f4"), ("ux", "<f4"), ("uy", "<f4"), ("v", "<f4"), ("vx", "<f4"), ("vy", "<f4"),
    ("u0", "<f4"), ("v0", "<f4"), ("zncc", "<f4"), ("iteration", "<f4"), ("convergence", "<f4"),
    ("feature", "<f4"),
])
assert POI_DTYPE.itemsize == 56


class DicConfig(ctypes.Structure):
    _fields_ = [("subset_radius_x", ctypes.c_int32), ("subset_radius_y", ctypes.c_int32),
                ("conv_criterion", ctypes.c_float), ("max_iteration", ctypes.c_int32),
                ("device", ctypes.c_int32), ("input_scale", ctypes.c_float)]


class DicFramePolicy(ctypes.Structure):
    _fields_ = [("skip_fftcc", ctypes.c_int32), ("poi_fallback", ctypes.c_int32),
                ("zncc_threshold", ctypes.c_float), ("frame_fallback_ratio", ctypes.c_float),
                ("learned_seed", ctypes.c_int32), ("temporal_extrapolation", ctypes.c_int32)]


class DicFrameReport(ctypes.Structure):
    _fields_ = [("pois", ctypes.c_int64), ("bad_before_repair", ctypes.c_int64),
                ("bad_after_repair", ctypes.c_int64), ("repaired_candidates", ctypes.c_int64),
                ("frame_fallback_used", ctypes.c_int32), ("fftcc_used", ctypes.c_int32),
                ("iteration_mean", ctypes.c_double), ("repaired_recovered", ctypes.c_int64),
                ("temporal_seed_count", ctypes.c_int64)]


class DicJob(ctypes.Structure):
    _fields_ = [("ref", ctypes.c_void_p), ("tar", ctypes.c_void_p), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32), ("row_stride_bytes", ctypes.c_int64), ("dtype", ctypes.c_int32),
                ("subset_radius", ctypes.c_int32), ("pois", ctypes.c_void_p), ("count", ctypes.c_int64)]


class DicBatchReport(ctypes.Structure):
    _fields_ = [("pois", ctypes.c_int64), ("valid", ctypes.c_int64), ("jobs", ctypes.c_int32),
                ("graph", ctypes.c_int32)]


class DicLaunchShape(ctypes.Structure):
    _fields_ = [("warps_per_cta", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("tuned", ctypes.c_int32),
                ("ms", ctypes.c_float), ("tile", ctypes.c_int32), ("warps_per_poi", ctypes.c_int32)]


class DicTuning(ctypes.Structure):
    _fields_ = [("icgn", DicLaunchShape * 5), ("batch", DicLaunchShape * 5)]


class DicStats(ctypes.Structure):
    _fields_ = [("ms_prepare_ref", ctypes.c_double), ("ms_poi_prepare", ctypes.c_double),
                ("ms_prepare_tar", ctypes.c_double), ("ms_fftcc", ctypes.c_double),
                ("ms_icgn", ctypes.c_double), ("ms_frame", ctypes.c_double), ("ms_proposal", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64),
                ("icgn_pois", ctypes.c_int64), ("icgn_iterations", ctypes.c_int64)]


# Every exported symbol with (restype, argtypes); tests check the .so exports all of them.
_vp = ctypes.c_void_p
_i32, _i64 = ctypes.c_int32, ctypes.c_int64
SIGNATURES = {
    "dic_version": (ctypes.c_char_p, []),
    "dic_abi_version": (_i32, []),
    "dic_device_info": (ctypes.c_int, [_i32, ctypes.c_char_p, _i32, ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                                       ctypes.POINTER(_i32), ctypes.POINTER(_i32)]),
    "dic_engine_create": (ctypes.c_int, [ctypes.POINTER(DicConfig), ctypes.POINTER(_vp)]),
    "dic_engine_destroy": (None, [_vp]),
    "dic_last_error": (ctypes.c_char_p, [_vp]),
    "dic_stream": (_vp, [_vp]),
    "dic_set_ref": (ctypes.c_int, [_vp, _vp, _i32, _i32, _i64, _i32]),
    "dic_set_tar": (ctypes.c_int, [_vp, _vp, _i32, _i32, _i64, _i32]),
    "dic_set_ref_device": (ctypes.c_int, [_vp, _vp, _i32, _i32, _i64, _i32]),
    "dic_set_tar_device": (ctypes.c_int, [_vp, _vp, _i32, _i32, _i64, _i32]),
    "dic_prepare_ref": (ctypes.c_int, [_vp, _vp, _i64]),
    "dic_prepare_tar": (ctypes.c_int, [_vp]),
    "dic_fftcc": (ctypes.c_int, [_vp, _vp, _i64, _vp]),
    "dic_icgn": (ctypes.c_int, [_vp, _vp, _i64]),
    "dic_process_pair": (ctypes.c_int, [_vp, _vp, _i64]),
    "dic_process_frame": (ctypes.c_int, [_vp, _vp, _i64, _vp, ctypes.POINTER(DicFramePolicy),
                                         ctypes.POINTER(DicFrameReport)]),
    "dic_process_frame_history": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp, ctypes.POINTER(DicFramePolicy),
                                                 ctypes.POINTER(DicFrameReport)]),
    "dic_run_device": (ctypes.c_int, [_vp, _vp, _i64, _i32]),
    "dic_process_pair_multi": (ctypes.c_int, [ctypes.POINTER(_vp), _i32, _vp, _i64, _vp]),
    "dic_split_rows": (ctypes.c_int, [_vp, _i64, _i32, _vp]),
    "dic_sequence_begin": (ctypes.c_int, [_vp, _vp, _i64, ctypes.POINTER(DicFramePolicy)]),
    "dic_stage_frame": (ctypes.c_int, [_vp, _vp, _i32, _i32, _i64, _i32]),
    "dic_sequence_frame": (ctypes.c_int, [_vp, _vp, _i32, _i32, _i64, _i32, _i32, _vp,
                                          ctypes.POINTER(DicFrameReport)]),
    "dic_sequence_fetch": (ctypes.c_int, [_vp, _i32, _vp, ctypes.POINTER(DicFrameReport)]),
    "dic_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(_vp)]),
    "dic_host_free": (None, [_vp]),
    "dic_set_graphs": (ctypes.c_int, [_vp, _i32]),
    "dic_batch_process": (ctypes.c_int, [_vp, ctypes.POINTER(DicJob), _i32, _i32, ctypes.POINTER(DicBatchReport)]),
    "dic_set_autotune": (ctypes.c_int, [_vp, _i32]),
    "dic_get_tuning": (ctypes.c_int, [_vp, ctypes.POINTER(DicTuning)]),
    "dic_set_launch_shape": (ctypes.c_int, [_vp, _i32, ctypes.POINTER(DicLaunchShape)]),
    "dic_set_sampling": (ctypes.c_int, [_vp, _i32]),
    "dic_read_plane": (ctypes.c_int, [_vp, _i32, _vp, _i64]),
    "dic_get_stats": (ctypes.c_int, [_vp, ctypes.POINTER(DicStats)]),
    "dic_set_timing": (ctypes.c_int, [_vp, _i32]),
    "dic_read_probe": (ctypes.c_int, [_i32, _vp, _i64, _i32, _vp, _vp]),
    "dic_fma_probe": (ctypes.c_int, [_i32, _i32, _vp, _vp, ctypes.POINTER(_i64)]),
    "dic_smem_probe": (ctypes.c_int, [_i32, _i32, _vp, _vp, ctypes.POINTER(_i64)]),
    "dic_cnn_param_count": (_i64, []),
    "dic_cnn_create": (ctypes.c_int, [_i32, ctypes.POINTER(_vp)]),
    "dic_cnn_destroy": (None, [_vp]),
    "dic_cnn_last_error": (ctypes.c_char_p, [_vp]),
    "dic_cnn_set_params": (ctypes.c_int, [_vp, _vp, _i64]),
    "dic_cnn_get_params": (ctypes.c_int, [_vp, _vp, _i64]),
    "dic_cnn_input": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _vp, _i64, _vp]),
    "dic_cnn_forward": (ctypes.c_int, [_vp, _vp, _i64, _vp]),
    "dic_cnn_seed": (ctypes.c_int, [_vp, _vp, _vp, _i32, _i32, _vp, _i64]),
    "dic_cnn_gradient": (ctypes.c_int, [_vp, _vp, _vp, _i64, _vp, ctypes.POINTER(ctypes.c_float)]),
    "dic_cnn_train_step": (ctypes.c_int, [_vp, _vp, _vp, _i64, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]),
    "dic_set_proposal": (ctypes.c_int, [_vp, _vp]),
    "dic_process_pair_learned": (ctypes.c_int, [_vp, _vp, _i64, ctypes.POINTER(DicFrameReport)]),
    "dic_process_pair_noalloc": (ctypes.c_int, [ctypes.POINTER(DicConfig), _vp, _vp, _i32, _i32, _i32, _vp, _i64,
                                                _vp, ctypes.c_char_p, _i64]),
}

_lib = None


def load(path: Path | None = None):
    """Load libdic.so and declare every signature.  Raises if the library is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -m fasticgn_gb300._build` "
                           "(the DIC engine has no CPU fallback)")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class DicError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


def raise_for(code: int, handle) -> None:
    """Map a dic_status to the exception the reference C++ classes throw."""
    if code == DIC_OK:
        return
    msg = load().dic_last_error(handle)
    msg = msg.decode() if msg else ""
    if code == DIC_ERR_ARGUMENT:
        raise ValueError(msg)              # std::invalid_argument
    if code == DIC_ERR_RANGE:
        raise IndexError(msg)              # std::out_of_range
    if code == DIC_ERR_STATE:
        raise RuntimeError(msg)            # std::logic_error
    raise DicError(code, msg)

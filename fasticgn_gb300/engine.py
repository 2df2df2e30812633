"""Python face of the GB300 DIC engine, mirroring the reference's solver classes.

``ICGN2D1`` mirrors ICGN2D1CudaMvp / OpenCorr ICGN2D1 (src/icgn2d1_cuda_mvp.h:98-143,
src/oc_icgn.h:45-77) and ``FFTCC2D`` mirrors FFTCC2DCuda / FFTCC2D (src/fftcc2d_cuda.h:85-109,
src/oc_fftcc.h:56-100): same constructor arguments, the same set / prepare / compute verbs
over a POI queue, and the same exceptions (ValueError for std::invalid_argument,
IndexError for std::out_of_range, RuntimeError for std::logic_error).  A POI queue is a
numpy structured array of ``POI_DTYPE`` (struct dic_poi).  ``Engine`` is the direct handle
on one dic_engine; both classes hold one.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import POI_DTYPE, DicConfig, DicStats

_DTYPES = {np.dtype(np.uint8): _lib.DIC_U8, np.dtype(np.uint16): _lib.DIC_U16,
           np.dtype(np.float32): _lib.DIC_F32}


def make_queue(xs, ys) -> np.ndarray:
    q = np.zeros(len(xs), dtype=POI_DTYPE)
    q["x"] = xs
    q["y"] = ys
    return q


def grid_queue(width: int, height: int, radius: int, step: int, lines=None) -> np.ndarray:
    """buildPoiQueue (opencorr_cli_cuda_mvp.cpp:2439-2472): margin r+2, y outer, x inner;
    with ``lines`` only those rows (in the order given, edge rows skipped)."""
    margin = radius + 2
    xs_line = np.arange(margin, width - margin, step, dtype=np.float32)
    if lines:
        rows = [y for y in lines if margin <= y < height - margin]
    else:
        rows = list(range(margin, height - margin, step))
    xs = np.tile(xs_line, len(rows))
    ys = np.repeat(np.asarray(rows, dtype=np.float32), len(xs_line))
    return make_queue(xs, ys)


def _check_queue(q: np.ndarray) -> np.ndarray:
    if not isinstance(q, np.ndarray) or q.dtype != POI_DTYPE or q.ndim != 1:
        raise TypeError("a POI queue is a 1-D numpy array of POI_DTYPE")
    if not q.flags.c_contiguous:
        raise ValueError("POI queue must be C-contiguous")
    return q


class Engine:
    """One dic_engine: one GPU, one stream, resident reference state."""

    def __init__(self, subset_radius_x: int, subset_radius_y: int | None = None,
                 conv_criterion: float = 0.001, max_iteration: int = 10, device: int = 0,
                 input_scale: float = 1.0):
        self._L = _lib.load()
        cfg = DicConfig(int(subset_radius_x), int(subset_radius_y if subset_radius_y is not None else subset_radius_x),
                        float(conv_criterion), int(max_iteration), int(device), float(input_scale))
        h = ctypes.c_void_p()
        rc = self._L.dic_engine_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != _lib.DIC_OK:
            if rc == _lib.DIC_ERR_ARGUMENT:
                raise ValueError("invalid DIC engine configuration")
            raise _lib.DicError(rc, "dic_engine_create failed (is a CUDA device available?)")
        self._h = h
        self.config = cfg

    # ------------------------------------------------------------------ lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.dic_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, rc: int) -> None:
        _lib.raise_for(rc, self._h)

    @property
    def stream(self) -> int:
        return int(self._L.dic_stream(self._h) or 0)

    # ------------------------------------------------------------------ images
    @staticmethod
    def _image(img: np.ndarray):
        img = np.asarray(img)
        if img.ndim != 2 or img.dtype not in _DTYPES:
            raise ValueError("an image is a 2-D uint8, uint16 or float32 array")
        if img.strides[1] != img.itemsize:
            img = np.ascontiguousarray(img)
        return img, _DTYPES[img.dtype]

    def set_ref(self, img: np.ndarray) -> None:
        img, dt = self._image(img)
        self._call(self._L.dic_set_ref(self._h, img.ctypes.data, img.shape[1], img.shape[0], img.strides[0], dt))

    def set_tar(self, img: np.ndarray) -> None:
        img, dt = self._image(img)
        self._call(self._L.dic_set_tar(self._h, img.ctypes.data, img.shape[1], img.shape[0], img.strides[0], dt))

    def set_ref_device(self, ptr: int, width: int, height: int, stride: int, dtype: int) -> None:
        self._call(self._L.dic_set_ref_device(self._h, ptr, width, height, stride, dtype))

    def set_tar_device(self, ptr: int, width: int, height: int, stride: int, dtype: int) -> None:
        self._call(self._L.dic_set_tar_device(self._h, ptr, width, height, stride, dtype))

    # ------------------------------------------------------------------ solvers
    def prepare_ref(self, queue: np.ndarray | None = None) -> None:
        if queue is None:
            self._call(self._L.dic_prepare_ref(self._h, None, 0))
        else:
            q = _check_queue(queue)
            self._call(self._L.dic_prepare_ref(self._h, q.ctypes.data, len(q)))

    def prepare_tar(self) -> None:
        self._call(self._L.dic_prepare_tar(self._h))

    def fftcc(self, queue: np.ndarray, cache_indices=None) -> np.ndarray:
        q = _check_queue(queue)
        idx_ptr = None
        if cache_indices is not None:
            idx = np.ascontiguousarray(cache_indices, dtype=np.int64)
            if idx.shape != (len(q),):
                raise ValueError("FFTCC2D::compute requires one cache index per POI")
            idx_ptr = idx.ctypes.data
        self._call(self._L.dic_fftcc(self._h, q.ctypes.data, len(q), idx_ptr))
        return q

    def icgn(self, queue: np.ndarray) -> np.ndarray:
        q = _check_queue(queue)
        self._call(self._L.dic_icgn(self._h, q.ctypes.data, len(q)))
        return q

    def process_pair(self, queue: np.ndarray) -> np.ndarray:
        q = _check_queue(queue)
        self._call(self._L.dic_process_pair(self._h, q.ctypes.data, len(q)))
        return q

    def process_frame(self, queue: np.ndarray, prev: np.ndarray | None, skip_fftcc: bool = True,
                      poi_fallback: bool = True, zncc_threshold: float = 0.8,
                      frame_fallback_ratio: float = float("inf"), prev_prev: np.ndarray | None = None,
                      temporal_extrapolation: bool = False):
        """processFrame: ``prev_prev`` (the frame before ``prev``) feeds the temporal
        extrapolation seed when ``temporal_extrapolation`` is set."""
        q = _check_queue(queue)
        ptrs = []
        for h in (prev, prev_prev):
            if h is None:
                ptrs.append(None)
                continue
            h = _check_queue(h)
            if len(h) != len(q):
                raise ValueError("previous results must have one record per POI")
            ptrs.append(h.ctypes.data)
        pol = _lib.DicFramePolicy(int(skip_fftcc), int(poi_fallback), float(zncc_threshold),
                                  float(frame_fallback_ratio), 0, int(bool(temporal_extrapolation)))
        rep = _lib.DicFrameReport()
        self._call(self._L.dic_process_frame_history(self._h, q.ctypes.data, len(q), ptrs[0], ptrs[1],
                                                     ctypes.byref(pol), ctypes.byref(rep)))
        return q, {f: getattr(rep, f) for f, _ in rep._fields_}

    def sequence_begin(self, template: np.ndarray, skip_fftcc: bool = True, poi_fallback: bool = True,
                       zncc_threshold: float = 0.8, frame_fallback_margin: float = 0.03,
                       learned_seed: bool = False, temporal_extrapolation: bool = False) -> None:
        """learned_seed: every frame seeded by the attached proposal network (IC-GN capped at
        6 iterations, FFTCC + IC-GN below ZNCC 0.9) instead of FFTCC / the previous frame.
        temporal_extrapolation: skip-FFTCC frames seed u, v from the previous two results."""
        q = _check_queue(template)
        pol = _lib.DicFramePolicy(int(skip_fftcc), int(poi_fallback), float(zncc_threshold),
                                  float(frame_fallback_margin), int(bool(learned_seed)),
                                  int(bool(temporal_extrapolation)))
        self._call(self._L.dic_sequence_begin(self._h, q.ctypes.data, len(q), ctypes.byref(pol)))
        self._seq_n = len(q)

    def stage_frame(self, img: np.ndarray) -> None:
        """Start the upload of the next frame on the engine's upload stream (see
        sequence_frame(staged=True))."""
        img, dt = self._image(img)
        self._call(self._L.dic_stage_frame(self._h, img.ctypes.data, img.shape[1], img.shape[0], img.strides[0], dt))

    def sequence_frame(self, tar, results: np.ndarray | None = None, device_ptr: int | None = None,
                       width: int = 0, height: int = 0, dtype: int = _lib.DIC_U8, staged: bool = False,
                       report: bool = True):
        """Solve one target frame of the sequence; ``tar`` is a host image, or None with
        ``device_ptr`` (dense rows) for a frame already on the device, or None with
        ``staged`` for the oldest frame passed to stage_frame."""
        rep = _lib.DicFrameReport()
        rep_ptr = ctypes.byref(rep) if report else None   # no report and no results: no host sync
        out_ptr = None
        if results is not None:
            results = _check_queue(results)
            if len(results) != self._seq_n:
                raise ValueError("results must hold one record per template POI")
            out_ptr = results.ctypes.data
        if staged:
            es = {_lib.DIC_U8: 1, _lib.DIC_U16: 2, _lib.DIC_F32: 4}[dtype]
            rc = self._L.dic_sequence_frame(self._h, None, width, height, width * es, dtype, _lib.DIC_PIXELS_STAGED,
                                            out_ptr, rep_ptr)
        elif tar is not None:
            img, dt = self._image(tar)
            rc = self._L.dic_sequence_frame(self._h, img.ctypes.data, img.shape[1], img.shape[0], img.strides[0], dt,
                                            0, out_ptr, rep_ptr)
        else:
            es = {_lib.DIC_U8: 1, _lib.DIC_U16: 2, _lib.DIC_F32: 4}[dtype]
            rc = self._L.dic_sequence_frame(self._h, device_ptr, width, height, width * es, dtype, 1, out_ptr,
                                            rep_ptr)
        self._call(rc)
        return {f: getattr(rep, f) for f, _ in rep._fields_} if report else None

    def sequence_fetch(self, results: np.ndarray | None = None, report: bool = True, frames_back: int = 0):
        """Results (and report) of an enqueued frame (frames_back 0: the most recent
        sequence_frame, 1: the one before), waiting only for that frame: a loop enqueues
        frame k + 1 with sequence_frame(..., report=False), stages frame k + 2, then fetches
        frame k with frames_back=1 while frame k + 1 runs."""
        rep = _lib.DicFrameReport()
        out_ptr = None
        if results is not None:
            results = _check_queue(results)
            if len(results) != self._seq_n:
                raise ValueError("results must hold one record per template POI")
            out_ptr = results.ctypes.data
        self._call(self._L.dic_sequence_fetch(self._h, int(frames_back), out_ptr, ctypes.byref(rep) if report else None))
        return {f: getattr(rep, f) for f, _ in rep._fields_} if report else None

    def set_proposal(self, net) -> None:
        """Attach a ProposalNet (or None) for process_pair_learned / DIC_RUN_LEARNED."""
        self._proposal = net
        self._call(self._L.dic_set_proposal(self._h, net.handle if net is not None else None))

    def process_pair_learned(self, queue: np.ndarray):
        q = _check_queue(queue)
        rep = _lib.DicFrameReport()
        self._call(self._L.dic_process_pair_learned(self._h, q.ctypes.data, len(q), ctypes.byref(rep)))
        return q, {f: getattr(rep, f) for f, _ in rep._fields_}

    def batch_process(self, jobs):
        """Uneven batch: jobs is a list of (ref, tar, subset_radius, queue) with host images
        (uint8 / uint16 / float32) and POI queues; queues are updated in place."""
        arr = (_lib.DicJob * len(jobs))()
        keep = []
        for k, (ref, tar, radius, queue) in enumerate(jobs):
            r, dt = self._image(ref)
            t, dt2 = self._image(tar)
            if r.shape != t.shape or dt != dt2 or r.strides != t.strides:
                raise ValueError("reference and target of a job must have the same size, type and layout")
            q = _check_queue(queue)
            keep += [r, t, q]
            arr[k] = _lib.DicJob(r.ctypes.data, t.ctypes.data, r.shape[1], r.shape[0], r.strides[0], dt, int(radius),
                                 q.ctypes.data, len(q))
        return self._batch(arr, len(jobs), 0)

    def batch_process_device(self, jobs):
        """Uneven batch with device-resident data: jobs is a list of (ref, tar, subset_radius,
        queue) torch CUDA tensors -- 2-D uint8 / uint16 / float32 images and a uint8 tensor of
        dic_poi records, updated in place.  Repeating the same jobs replays a CUDA graph."""
        import torch
        tdt = {torch.uint8: _lib.DIC_U8, torch.int16: _lib.DIC_U16, torch.float32: _lib.DIC_F32}
        if hasattr(torch, "uint16"):
            tdt[torch.uint16] = _lib.DIC_U16
        arr = (_lib.DicJob * len(jobs))()
        rec = POI_DTYPE.itemsize
        for k, (ref, tar, radius, queue) in enumerate(jobs):
            if ref.shape != tar.shape or ref.dtype != tar.dtype or ref.dim() != 2 or ref.stride(1) != 1 \
                    or tar.stride() != ref.stride():
                raise ValueError("reference and target of a job must have the same size, type and layout")
            if queue.dtype != torch.uint8 or queue.numel() % rec or not queue.is_contiguous():
                raise ValueError("a device queue is a contiguous uint8 tensor of dic_poi records")
            arr[k] = _lib.DicJob(ref.data_ptr(), tar.data_ptr(), ref.shape[1], ref.shape[0],
                                 ref.stride(0) * ref.element_size(), tdt[ref.dtype], int(radius), queue.data_ptr(),
                                 queue.numel() // rec)
        torch.cuda.synchronize()
        return self._batch(arr, len(jobs), 1)

    def _batch(self, arr, n, on_device):
        rep = _lib.DicBatchReport()
        self._call(self._L.dic_batch_process(self._h, arr, n, on_device, ctypes.byref(rep)))
        return {f: getattr(rep, f) for f, _ in rep._fields_}

    def set_autotune(self, enabled: bool) -> None:
        self._call(self._L.dic_set_autotune(self._h, int(bool(enabled))))

    def tuning(self) -> dict:
        t = _lib.DicTuning()
        self._call(self._L.dic_get_tuning(self._h, ctypes.byref(t)))

        def shape(s):
            return {f: getattr(s, f) for f, _ in s._fields_}
        return {"icgn_flat": shape(t.icgn[0]), "icgn_column": shape(t.icgn[1]), "icgn_pair": shape(t.icgn[2]),
                "icgn_column_px": shape(t.icgn[3]), "icgn_pair_px": shape(t.icgn[4]),
                "batch_flat": shape(t.batch[0]), "batch_column": shape(t.batch[1]), "batch_pair": shape(t.batch[2]),
                "batch_column_px": shape(t.batch[3]), "batch_pair_px": shape(t.batch[4])}

    WALK_FLAT, WALK_COLUMN, WALK_PAIR, WALK_COLUMN_PX, WALK_PAIR_PX = 0, 1, 2, 3, 4

    def set_sampling(self, mode: int) -> None:
        """How IC-GN reads the target (dic_set_sampling): DIC_SAMPLE_PIXELS (default; the
        bicubic polynomial from the 4 x 4 pixels, windows staged in shared memory) or
        DIC_SAMPLE_TABLE (BicubicBspline's coefficient table)."""
        self._call(self._L.dic_set_sampling(self._h, int(mode)))

    def set_launch_shape(self, walk: int, warps_per_cta: int = 4, ctas_per_sm: int = 0, tile: int = 0,
                         warps_per_poi: int = 1) -> None:
        """Fixes the single-queue IC-GN launch of one subset walk (dic_set_launch_shape): walk 1
        column (subsets up to 32 wide), 2 pair (33 to 64), 0 flat (wider), 3 and 4 column and
        pair under pixel sampling; ``tile`` 1 or 2 selects the TMA-staged coefficient tile forms
        (walk 1), with walks 3 and 4 ``tile`` 1 stages pixel windows by TMA, 2 by warp copies and
        0 reads the global plane; ``warps_per_poi`` 2 the two-warp pair walks.  A bool walk is
        read as column (True) or flat (False)."""
        s = _lib.DicLaunchShape(warps_per_cta, ctas_per_sm, 0, 0.0, tile, warps_per_poi)
        self._call(self._L.dic_set_launch_shape(self._h, int(walk), ctypes.byref(s)))

    def set_graphs(self, enabled: bool) -> None:
        self._call(self._L.dic_set_graphs(self._h, int(bool(enabled))))

    def run_device(self, device_pois: int, count: int, flags: int) -> None:
        self._call(self._L.dic_run_device(self._h, device_pois, count, flags))

    def read_plane(self, plane: int, width: int, height: int) -> np.ndarray:
        """A resident plane; the coefficient table comes back as [row k][y][x][4] (its device
        layout is two planes of rows 0-1 and 2-3 per texel)."""
        shape = {_lib.DIC_PLANE_REF: (height, width), _lib.DIC_PLANE_TAR: (height, width),
                 _lib.DIC_PLANE_REF_PACK: (height, width, 4), _lib.DIC_PLANE_TAR_COEF: (2, height, width, 2, 4)}[plane]
        out = np.empty(shape, dtype=np.float32)
        self._call(self._L.dic_read_plane(self._h, plane, out.ctypes.data, out.nbytes))
        if plane == _lib.DIC_PLANE_TAR_COEF:
            out = np.ascontiguousarray(out.transpose(0, 3, 1, 2, 4).reshape(4, height, width, 4))
        return out

    def set_timing(self, enabled: bool) -> None:
        self._call(self._L.dic_set_timing(self._h, int(bool(enabled))))

    def stats(self) -> dict:
        s = DicStats()
        self._call(self._L.dic_get_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}


def split_rows(queue: np.ndarray, parts: int) -> np.ndarray:
    """Row-band partition of a queue (dic_split_rows): parts + 1 boundaries, every inner one at
    the first change of y at or after k * len / parts, so no row of POIs is split."""
    q = _check_queue(queue)
    starts = np.zeros(int(parts) + 1, dtype=np.int64)
    rc = _lib.load().dic_split_rows(q.ctypes.data, len(q), int(parts), starts.ctypes.data)
    if rc != _lib.DIC_OK:
        raise ValueError("split_rows: bad arguments")
    return starts


def process_pair_multi(engines, queue: np.ndarray) -> np.ndarray:
    """One pair over several engines (one per GPU), each solving a row band of the queue from
    its own host thread (dic_process_pair_multi); the queue is updated in place, in queue
    order.  Returns the band boundaries."""
    q = _check_queue(queue)
    arr = (ctypes.c_void_p * len(engines))(*[e._h for e in engines])
    starts = np.zeros(len(engines) + 1, dtype=np.int64)
    rc = _lib.load().dic_process_pair_multi(arr, len(engines), q.ctypes.data, len(q), starts.ctypes.data)
    if rc != _lib.DIC_OK:
        failed = next((e for e in engines if _lib.load().dic_last_error(e._h)), engines[0])
        _lib.raise_for(rc, failed._h)
    return starts


class ICGN2D1:
    """ICGN2D1CudaMvp(rx, ry, conv_criterion, stop_condition, device) on the GB300 engine."""

    def __init__(self, subset_radius_x: int, subset_radius_y: int, conv_criterion: float = 0.001,
                 stop_condition: int = 10, device: int = 0, input_scale: float = 1.0):
        self.engine = Engine(subset_radius_x, subset_radius_y, conv_criterion, int(stop_condition), device,
                             input_scale)

    def setImages(self, ref_img, tar_img):
        self.setRefImage(ref_img)
        self.setTarImage(tar_img)

    def setRefImage(self, ref_img):
        self.engine.set_ref(ref_img)

    def setTarImage(self, tar_img):
        self.engine.set_tar(tar_img)

    def prepareRef(self, poi_queue: np.ndarray | None = None):
        self.engine.prepare_ref(poi_queue)

    def prepareTar(self):
        self.engine.prepare_tar()

    def prepare(self):
        self.prepareRef()
        self.prepareTar()

    def compute(self, poi_queue: np.ndarray) -> np.ndarray:
        return self.engine.icgn(poi_queue)


class FFTCC2D:
    """FFTCC2DCuda(rx, ry, device) on the GB300 engine (square radii only, as the reference)."""

    def __init__(self, subset_radius_x: int, subset_radius_y: int, device: int = 0, input_scale: float = 1.0):
        if subset_radius_x <= 0 or subset_radius_x != subset_radius_y or subset_radius_x > 23170:
            raise ValueError("FFTCC2D supports positive square radii only (1..23170); "
                             "rectangular FFTs are unsupported")
        self.engine = Engine(subset_radius_x, subset_radius_y, device=device, input_scale=input_scale)

    def setImages(self, ref_img, tar_img):
        self.setRefImage(ref_img)
        self.setTarImage(tar_img)

    def setRefImage(self, ref_img):
        self.engine.set_ref(ref_img)

    def setTarImage(self, tar_img):
        self.engine.set_tar(tar_img)

    def prepareRef(self, poi_queue: np.ndarray):
        self.engine.prepare_ref(poi_queue)

    def prepareTar(self):
        self.engine.prepare_tar()

    def compute(self, poi_queue: np.ndarray, cache_indices=None) -> np.ndarray:
        return self.engine.fftcc(poi_queue, cache_indices)

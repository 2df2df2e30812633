#!/usr/bin/env python3
"""Throughput of the FFTCC-seeded first-order IC-GN path on one GB300.

Workload (one step = one image pair solved end to end): 2048x2048 u8 synthetic speckle, the
target warped by a smooth field (8 Gaussian bumps per component, |u|,|v| up to ~10 px,
local strain up to 2 %, noise 2 DN); subset radius 15, POI grid step 4 with margin r+2
(254 016 POIs).  A step runs reference prep (float plane, Gradient2D4 planes, per-POI
mean/norm/inverse Hessian), target prep (B-spline table), FFTCC and IC-GN.

value  = POIs / device time per step, inputs resident in HBM (dic_run_device), L2 flushed
         (256 MB write) before every timed step, CUDA events on the engine stream.
e2e    = the same through the C ABI with host buffers (dic_set_ref / dic_set_tar /
         dic_process_pair): pinned host images and POI queue copied in, results copied out.
--impl reference: the reference's CPU path (the oracle restatement, all host threads) on the
         whole queue of the same pair, every step.
roofline: the IC-GN gathers are served by L2, so their bound is the L2-to-SM read bandwidth,
         measured in the same run by dic_read_probe (the gathers' 256-bit loads over an
         L2-resident buffer); the DRAM side is reported beside it.
"""
from __future__ import annotations

import argparse
import ctypes
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = {"name": "pair2048_bumps_r15_step4", "width": 2048, "height": 2048, "radius": 15, "step": 4,
            "seed": 4, "conv": 0.001, "max_iter": 10}
L2_FLUSH_BYTES = 256 << 20
STREAM_PARITY_STRIDE = 8        # every 8th POI of a stream frame is re-solved by the CPU oracle


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def load_pair():
    """The synthetic pair, cached per process tree under $DIC_BENCH_CACHE (default /tmp)."""
    from fasticgn_gb300 import speckle
    cache = Path(os.environ.get("DIC_BENCH_CACHE", "/tmp")) / f"gb300_dic_{WORKLOAD['name']}_v1.npz"
    if cache.exists():
        d = np.load(cache)
        return d["ref"], d["tar"]
    t = time.time()
    pr = speckle.pair_bumps(seed=WORKLOAD["seed"], width=WORKLOAD["width"], height=WORKLOAD["height"])
    log(f"generated workload in {time.time() - t:.1f} s")
    try:
        tmp = cache.with_suffix(f".tmp{os.getpid()}.npz")
        np.savez(tmp, ref=pr.ref, tar=pr.tar)
        os.replace(tmp, cache)
    except OSError:
        pass
    return pr.ref, pr.tar


UNEVEN = {"name": "uneven16_r10-30", "seed": 3, "count": 16}


def load_uneven():
    """The uneven batch (16 pairs, sides 256..4096, radii {10,15,20,30}, 1k..600k POIs each,
    20 % flat patches), rendered on all host cores and cached like the pair."""
    from fasticgn_gb300 import speckle
    cache = Path(os.environ.get("DIC_BENCH_CACHE", "/tmp")) / f"gb300_dic_{UNEVEN['name']}_v1.npz"
    if cache.exists():
        d = np.load(cache)
        n = int(d["count"])
        return [(d[f"ref{k}"], d[f"tar{k}"], int(d["radius"][k]), int(d["step"][k])) for k in range(n)]
    t = time.time()
    specs = speckle.uneven_specs(seed=UNEVEN["seed"], count=UNEVEN["count"])
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(min(len(specs), os.cpu_count() or 1)) as pool:
        jobs = pool.map(speckle.render_uneven_job, specs, chunksize=1)
    log(f"generated uneven batch in {time.time() - t:.1f} s")
    try:
        tmp = cache.with_suffix(f".tmp{os.getpid()}.npz")
        arrays = {"count": np.int64(len(jobs)), "radius": np.array([j[2] for j in jobs]),
                  "step": np.array([j[3] for j in jobs])}
        for k, j in enumerate(jobs):
            arrays[f"ref{k}"], arrays[f"tar{k}"] = j[0], j[1]
        np.savez(tmp, **arrays)
        os.replace(tmp, cache)
    except OSError:
        pass
    return jobs


STREAMS = [
    # 12-bit 2048x2048 sine/strain stream, skip-FFTCC seeding from the previous frame; 64
    # consecutive frames from the middle of the 200-frame ramp
    {"name": "stream2048_12bit_r15_step5", "kind": "stream", "seed": 2, "width": 2048, "height": 2048,
     "frames": 200, "window": list(range(100, 164)), "radius": 15, "step": 5, "learned": False},
    # 12-bit 1024x1024 crack stream, learned seed + FFTCC fallback on every frame; the last 48
    # frames of the 5000-frame ramp (crack jump 1.49-1.5 px)
    {"name": "crack1024_12bit_r12_step4", "kind": "crack", "seed": 5, "width": 1024, "height": 1024,
     "frames": 5000, "window": list(range(4952, 5000)), "radius": 12, "step": 4, "learned": True},
]


def load_streams():
    """Reference + window frames of each stream, rendered on all host cores, cached."""
    from fasticgn_gb300 import speckle
    out, todo = {}, []
    for st in STREAMS:
        cache = Path(os.environ.get("DIC_BENCH_CACHE", "/tmp")) / f"gb300_dic_{st['name']}_v2.npz"
        if cache.exists():
            d = np.load(cache)
            out[st["name"]] = (d["ref"], [d[f"f{k}"] for k in st["window"]])
        else:
            todo.append(st)
    if todo:
        t = time.time()
        specs = [(st["kind"], st["seed"], st["width"], st["height"], st["frames"], k)
                 for st in todo for k in [-1] + st["window"]]
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(min(len(specs), os.cpu_count() or 1)) as pool:
            imgs = pool.map(speckle.stream_image, specs, chunksize=1)
        log(f"generated streams in {time.time() - t:.1f} s")
        pos = 0
        for st in todo:
            n = 1 + len(st["window"])
            ref, frames = imgs[pos], imgs[pos + 1:pos + n]
            pos += n
            out[st["name"]] = (ref, frames)
            try:
                cache = Path(os.environ.get("DIC_BENCH_CACHE", "/tmp")) / f"gb300_dic_{st['name']}_v2.npz"
                tmp = cache.with_suffix(f".tmp{os.getpid()}.npz")
                np.savez(tmp, ref=ref, **{f"f{k}": f for k, f in zip(st["window"], frames)})
                os.replace(tmp, cache)
            except OSError:
                pass
    return out


def grid():
    from fasticgn_gb300 import grid_queue
    return grid_queue(WORKLOAD["width"], WORKLOAD["height"], WORKLOAD["radius"], WORKLOAD["step"])


# ------------------------------------------------------------------------------ CPU legs

def cpu_pair_time(ref, tar, threads):
    """Reference CPU path on the whole queue: full-image prep, FFTCC and IC-GN on every POI
    (OpenMP over POIs, src/oc_icgn.cpp:389-397, src/oc_fftcc.cpp:529-557).
    Returns (POIs/s, detail dict, results)."""
    from oracle import oracle as O
    w, h, r = WORKLOAD["width"], WORKLOAD["height"], WORKLOAD["radius"]
    reff, tarf = ref.astype(np.float32), tar.astype(np.float32)
    pois = O.grid_pois(w, h, r, WORKLOAD["step"])
    t0 = time.perf_counter()
    gx, gy = O.gradient(reff, threads)
    coef = O.bspline_prepare(tarf, threads)
    t1 = time.perf_counter()
    O.fftcc2d(reff, tarf, pois, r, threads)
    t2 = time.perf_counter()
    O.icgn2d1(reff, gx, gy, coef, pois, r, WORKLOAD["conv"], WORKLOAD["max_iter"], threads)
    t3 = time.perf_counter()
    detail = {"prep_s": t1 - t0, "fftcc_s": t2 - t1, "icgn_s": t3 - t2, "pois": len(pois), "pair_s": t3 - t0}
    return len(pois) / (t3 - t0), detail, pois


CPU_SAMPLE = ("the whole queue of the pair every step (254 016 POIs): full-image gradient + B-spline table, "
              "FFTCC and IC-GN on every POI, OpenMP over POIs on all host threads; own FFT, not FFTW")


def run_reference(args):
    from oracle import oracle as O
    threads = O.default_threads()
    ref, tar = load_pair()
    for _ in range(args.warmup):
        cpu_pair_time(ref, tar, threads)
    pair_s = []
    for _ in range(args.steps):
        _, d, _ = cpu_pair_time(ref, tar, threads)
        pair_s.append(d["pair_s"])
    value = d["pois"] * len(pair_s) / float(np.sum(pair_s))
    line = {"impl": "reference", "metric": "POIs/s", "value": value, "unit": "POI/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(pair_s)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_block(),
            "cpu_baseline": {"value": value, "unit": "POI/s", "cores": threads, "kind": "port", "sample": CPU_SAMPLE},
            "e2e": {"value": value, "unit": "POI/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_block():
    return {"workload": WORKLOAD["name"], "image": f"{WORKLOAD['width']}x{WORKLOAD['height']} u8 speckle",
            "field": "8 Gaussian bumps per component, |u|,|v| <= ~10 px, strain <= 2 %, noise 2 DN",
            "subset_radius": WORKLOAD["radius"], "poi_step": WORKLOAD["step"], "pois": len(grid()),
            "seed_method": "FFTCC", "conv_criterion": WORKLOAD["conv"], "max_iteration": WORKLOAD["max_iter"],
            "l2": "flushed before every timed step (256 MB device write, untimed)",
            "step": "ref prep + per-POI prep + target B-spline table + FFTCC + IC-GN"}


# ------------------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi every 50 ms for the whole run; the summary keeps the samples taken inside
    the timed regions (marked with window()), so the clock record belongs to the timing."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 50

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []        # (host time, csv line)
        self.windows = {}      # name -> [(t0, t1)]

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    class _Window:
        def __init__(self, owner, name):
            self.owner, self.name = owner, name

        def __enter__(self):
            self.t0 = time.perf_counter()

        def __exit__(self, *exc):
            # a sample is printed up to one period after it is taken
            self.owner.windows.setdefault(self.name, []).append(
                (self.t0, time.perf_counter() + self.owner.PERIOD_MS * 1e-3))

    def window(self, name: str):
        return self._Window(self, name)

    def summary(self, names=None):
        spans = [w for n, ws in self.windows.items() if names is None or n in names for w in ws]
        sm, smax, power, reasons = [], [], [], set()
        fields = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in self.lines:
            if not any(a <= t <= b for a, b in spans):
                continue
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(fields, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        timed_s = sum(b - a - self.PERIOD_MS * 1e-3 for a, b in spans)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0, "timed_s": timed_s}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "sm_mhz_min": min(sm), "power_w_max": max(power), "timed_s": timed_s,
                "period_ms": self.PERIOD_MS}


# ------------------------------------------------------------------------------ GPU arm

def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled(kernel: str):
    """ncu figures of one launch of a kernel on this workload (profiles/traffic.json):
    DRAM bytes per launch and the L2 (lts) throughput percentage, with their source."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return {}
    d = json.loads(p.read_text())
    k = d.get("kernels", {}).get(kernel)
    if not k or d.get("workload") != WORKLOAD["name"]:
        return {}
    return dict(k, source=d.get("source"))


def measure_read_peak(torch, dev):
    """L2-to-SM read bandwidth with the gathers' own load (dic_read_probe): a 64 MiB buffer
    that L2 (126 MB) holds, 40 passes per launch, best of 5 launches after 2 warm-ups, CUDA
    events on the probe's stream.  The same kernel over a 4 GiB buffer (one pass) gives the
    HBM read rate for comparison."""
    from fasticgn_gb300 import _lib
    L = _lib.load()
    stream = torch.cuda.Stream(device=dev)
    sink = torch.zeros(1, dtype=torch.float32, device=dev)
    out = {}
    for name, nbytes, repeats in (("l2", 64 << 20, 40), ("hbm", 4 << 30, 1)):
        buf = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        with torch.cuda.stream(stream):
            buf.random_(0, 255)
        best = None
        for k in range(7):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                s.record(stream)
                rc = L.dic_read_probe(dev.index, buf.data_ptr(), nbytes, repeats, sink.data_ptr(), stream.cuda_stream)
                e.record(stream)
            if rc != _lib.DIC_OK:
                raise RuntimeError(f"dic_read_probe failed ({rc})")
            e.synchronize()
            if k >= 2:
                ms = s.elapsed_time(e)
                best = ms if best is None else min(best, ms)
        out[name] = {"gbs": nbytes * repeats / (best * 1e-3) / 1e9, "bytes": nbytes, "passes": repeats,
                     "ms": best}
        del buf
    # FP32 FMA rate (the FFTCC kernels' bound), same timing
    flop = ctypes.c_int64(0)
    best = None
    for k in range(7):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            s.record(stream)
            rc = L.dic_fma_probe(dev.index, 1 << 16, sink.data_ptr(), stream.cuda_stream, ctypes.byref(flop))
            e.record(stream)
        if rc != _lib.DIC_OK:
            raise RuntimeError(f"dic_fma_probe failed ({rc})")
        e.synchronize()
        if k >= 2:
            ms = s.elapsed_time(e)
            best = ms if best is None else min(best, ms)
    out["fp32"] = {"tflops": flop.value / (best * 1e-3) / 1e12, "ms": best}
    # shared-memory load bandwidth (the pixel-sampled IC-GN's sample path), same timing
    nbytes = ctypes.c_int64(0)
    best = None
    for k in range(7):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            s.record(stream)
            rc = L.dic_smem_probe(dev.index, 1 << 12, sink.data_ptr(), stream.cuda_stream, ctypes.byref(nbytes))
            e.record(stream)
        if rc != _lib.DIC_OK:
            raise RuntimeError(f"dic_smem_probe failed ({rc})")
        e.synchronize()
        if k >= 2:
            ms = s.elapsed_time(e)
            best = ms if best is None else min(best, ms)
    out["smem"] = {"gbs": nbytes.value / (best * 1e-3) / 1e9, "bytes": nbytes.value, "ms": best}
    torch.cuda.synchronize()
    return out


def parity_vs_cpu(result, cpu_result):
    """Reference parity-gate statistics of GPU results against the CPU oracle's results on
    the same POIs (smoke/check_cpu_gpu_parity.py:46-98), plus flag agreement."""
    from oracle import oracle as O
    cz, gz = cpu_result["r"][:, O.R_ZNCC], result["zncc"]
    both = (cz >= 0) & (gz >= 0) & np.isfinite(cz) & np.isfinite(gz)
    du = np.abs(cpu_result["p"][both, O.P_U] - result["u"][both])
    dv = np.abs(cpu_result["p"][both, O.P_V] - result["v"][both])
    neg = lambda z: np.where(np.isfinite(z) & (z < 0), z, 0)   # noqa: E731
    return {"pois": int(len(result)), "shared_valid": int(both.sum()),
            "median_du": float(np.median(du)), "median_dv": float(np.median(dv)),
            "p99_du": float(np.quantile(du, 0.99)), "p99_dv": float(np.quantile(dv, 0.99)),
            "max_du": float(du.max()), "max_dv": float(dv.max()),
            "cpu_valid_gpu_valid_agreement": float(np.mean((cz >= 0) == (gz >= 0))),
            "failure_codes_identical": float(np.mean(neg(cz) == neg(gz)))}


def stream_parity(frame, tmpl, radius, result, stride=STREAM_PARITY_STRIDE):
    """A stream frame's GPU results against the CPU oracle solving the same frame from scratch
    (FFTCC + IC-GN) on every stride-th POI of the template: the converged IC-GN is the judge,
    whatever seed the stream used."""
    from oracle import oracle as O
    ref, tar = frame
    idx = np.arange(0, len(tmpl), stride)
    pois = O.make_pois(tmpl["x"][idx], tmpl["y"][idx])
    O.run_pair(ref.astype(np.float32), tar.astype(np.float32), pois, radius, WORKLOAD["conv"],
               WORKLOAD["max_iter"], threads=O.default_threads())
    out = parity_vs_cpu(result[idx], pois)
    out["sample"] = f"every {stride}th POI of the last timed frame, CPU FFTCC + IC-GN from scratch"
    return out


def measure_uneven(dic, torch, dev, flush, jobs, steps, warmup, clock):
    """The uneven batch through dic_batch_process with device-resident pairs and queues
    (graph replay after the first two calls, autotuned launch shapes), next to the same
    pairs run one at a time through the single-pair device entry point."""
    from fasticgn_gb300 import _lib
    tdt = {np.dtype(np.uint8): _lib.DIC_U8}
    eng = dic.Engine(15, 15, WORKLOAD["conv"], WORKLOAD["max_iter"], device=dev.index)
    eng.set_autotune(True)
    stream = torch.cuda.ExternalStream(eng.stream, device=dev)
    djobs, pristine = [], []
    for ref, tar, r, step in jobs:
        q = dic.grid_queue(ref.shape[1], ref.shape[0], r, step)
        qd = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
        pristine.append(qd.clone())
        djobs.append((torch.from_numpy(ref).to(dev), torch.from_numpy(tar).to(dev), r, qd))
    total = sum(p.numel() // dic.POI_DTYPE.itemsize for p in pristine)

    def reset():
        with torch.cuda.stream(stream):
            for (_, _, _, qd), p in zip(djobs, pristine):
                qd.copy_(p)
            flush.random_(0, 255)

    def timed(fn):
        reset()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        fn()
        e.record(stream)
        e.synchronize()
        return s.elapsed_time(e)

    eager_ms = []
    for _ in range(max(2, warmup)):          # the first call tunes, the second captures the graph
        eager_ms.append(timed(lambda: eng.batch_process_device(djobs)))
    launches0 = eng.stats()["kernel_launches"]
    with clock.window("uneven_batch"):
        graph_ms = [timed(lambda: eng.batch_process_device(djobs)) for _ in range(steps)]
    launches = (eng.stats()["kernel_launches"] - launches0) / steps
    batch_out = [qd.cpu().numpy().view(dic.POI_DTYPE).copy() for _, _, _, qd in djobs]

    # the same pairs one at a time (a per-pair engine per radius, dic_run_device per pair)
    engines = {}
    flags = _lib.DIC_RUN_FFTCC | _lib.DIC_RUN_ICGN | _lib.DIC_RUN_PREPARE

    def per_pair():
        for (ref_d, tar_d, r, qd) in djobs:
            e = engines.get(r)
            if e is None:
                e = engines[r] = dic.Engine(r, r, WORKLOAD["conv"], WORKLOAD["max_iter"], device=dev.index)
            h, w = ref_d.shape
            e.set_ref_device(ref_d.data_ptr(), w, h, w, tdt[np.dtype(np.uint8)])
            e.set_tar_device(tar_d.data_ptr(), w, h, w, tdt[np.dtype(np.uint8)])
            e.run_device(qd.data_ptr(), qd.numel() // dic.POI_DTYPE.itemsize, flags)
        torch.cuda.synchronize()

    for _ in range(2):
        reset()
        torch.cuda.synchronize()
        per_pair()
    # per-pair calls run on several engine streams: time them on the host around a full sync
    loop_ms = []
    for _ in range(max(3, steps // 4)):
        reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        per_pair()
        loop_ms.append(1e3 * (time.perf_counter() - t0))
    same = all(np.array_equal(a.view(np.uint8), qd.cpu().numpy())
               for a, (_, _, _, qd) in zip(batch_out, djobs))
    allq = np.concatenate(batch_out)
    ms = float(np.mean(graph_ms))
    out = {"workload": UNEVEN["name"], "pairs": len(jobs), "pois": int(total),
           "radii": sorted({int(j[2]) for j in jobs}),
           "pixels": int(sum(j[0].size for j in jobs)),
           "value": total / (ms * 1e-3), "unit": "POI/s", "ms_per_step": ms,
           "first_call_ms": eager_ms[0], "eager_ms": eager_ms[-1] if len(eager_ms) > 1 else None,
           "per_pair_loop_ms": float(np.median(loop_ms)),
           "speedup_vs_per_pair_loop": float(np.median(loop_ms)) / ms,
           "valid_ratio": float((allq["zncc"] >= 0).mean()),
           "icgn_iterations_per_poi": float(allq["iteration"].mean()),
           "kernel_launches_per_step": launches, "tuning": eng.tuning(),
           "matches_per_pair_path": bool(same),
           "timing": "graph replay, device-resident pairs and queues, L2 flushed before each step; "
                     "per-pair loop timed on the host around a device sync"}
    for e in engines.values():
        e.close()
    eng.close()
    return out


def measure_stream(dic, torch, dev, st, ref, tars, net, flush, clock):
    """A fixed-reference stream through dic_sequence_*: e2e = host frames staged on the side
    stream (dic_stage_frame) and every frame's results read back one frame behind the solve
    (dic_sequence_fetch), host clock, including the read of warm-up frame 1; device =
    frames already in HBM, back-to-back frames without host syncs, CUDA events.  Frames 0
    (first / FFTCC) and 1 (graph capture) of the window are untimed warm-up."""
    from fasticgn_gb300 import _lib, speckle
    W, H, R = st["width"], st["height"], st["radius"]
    tmpl = dic.grid_queue(W, H, R, st["step"])
    n = len(tmpl)
    learned = st["learned"] and net is not None
    eng = dic.Engine(R, R, WORKLOAD["conv"], WORKLOAD["max_iter"], device=dev.index)
    eng.set_autotune(True)
    if learned:
        eng.set_proposal(net)
    eng.set_ref(ref)
    stream = torch.cuda.ExternalStream(eng.stream, device=dev)
    # one pinned result buffer per frame, so that reading results back costs no extra copy
    res_all = torch.empty((len(tars), n * dic.POI_DTYPE.itemsize), dtype=torch.uint8).pin_memory().numpy()
    tars_h = [torch.from_numpy(t).pin_memory().numpy() for t in tars]

    # ---- e2e: staged host frames, results every frame
    eng.sequence_begin(tmpl, learned_seed=learned)
    reports, results = [], []
    def enqueue(k):
        eng.stage_frame(tars_h[k])
        eng.sequence_frame(None, None, staged=True, width=W, height=H, dtype=_lib.DIC_U16, report=False)

    t0 = None
    gc.disable()   # no collector pause inside a ~30 ms host-clocked window
    enqueue(0)
    win = clock.window(st["name"])
    for k in range(len(tars_h)):
        if k == 1:   # frames 0 and 1 solved; the clock covers staging, solving and reading 2..
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            win.__enter__()
        # frame k is running: stage frame k + 1 (upload on the side stream, straight from the
        # page-locked frame) and enqueue it behind frame k, then read frame k's results one
        # frame back while frame k + 1 runs, so the device never waits for the host
        ahead = k + 1 < len(tars_h)
        if ahead:
            enqueue(k + 1)
        res = res_all[k].view(dic.POI_DTYPE)
        rep = eng.sequence_fetch(res, frames_back=1 if ahead else 0)
        if k >= 2:
            reports.append(rep)
            results.append(res)
    e2e_s = time.perf_counter() - t0
    win.__exit__(None, None, None)
    gc.enable()
    timed = len(tars_h) - 2
    # ---- device-resident frames
    tars_d = [torch.from_numpy(t).to(dev) for t in tars]
    eng.sequence_begin(tmpl, learned_seed=learned)
    for k in range(2):
        eng.sequence_frame(None, device_ptr=tars_d[k].data_ptr(), width=W, height=H, dtype=_lib.DIC_U16)
    with torch.cuda.stream(stream):
        flush.random_(0, 255)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
    l0 = eng.stats()["kernel_launches"]
    with clock.window(st["name"]):
        for k in range(2, len(tars_d)):
            eng.sequence_frame(None, device_ptr=tars_d[k].data_ptr(), width=W, height=H, dtype=_lib.DIC_U16,
                               report=False)
        with torch.cuda.stream(stream):
            e.record(stream)
        e.synchronize()
    dev_ms = s.elapsed_time(e)
    launches = (eng.stats()["kernel_launches"] - l0) / timed
    allr = np.concatenate(results)
    out = {"workload": st["name"], "image": f"{W}x{H} 12-bit in u16", "subset_radius": R, "poi_step": st["step"],
           "pois_per_frame": n, "frames_timed": timed, "seed": "learned proposal + FFTCC fallback" if learned
           else "previous frame (skip-FFTCC), POI-level repair and whole-frame fallback",
           "window": [st["window"][0], st["window"][-1]], "ramp_frames": st["frames"],
           "frames_per_s": timed / e2e_s, "pois_per_s": timed * n / e2e_s,
           "device_frames_per_s": timed / (dev_ms * 1e-3), "device_pois_per_s": timed * n / (dev_ms * 1e-3),
           "kernel_launches_per_frame": launches,
           "valid_ratio": float((allr["zncc"] >= 0).mean()),
           "icgn_iterations_per_poi": float(allr["iteration"][allr["zncc"] >= 0].mean()),
           "fallback_rate": float(np.mean([r["repaired_candidates"] for r in reports]) / n),
           "frame_fallbacks": int(sum(r["frame_fallback_used"] for r in reports)),
           "tuning": eng.tuning(),
           "parity_vs_cpu": stream_parity((ref, tars[-1]), tmpl, R, results[-1]),
           "timing": "e2e: host clock over the timed frames, the next frame uploaded and enqueued while each "
                     "frame runs, every frame's results read one frame behind (uploads and result reads "
                     "included); "
                     "device: CUDA events on the engine stream, frames resident, no per-frame host sync"}
    if st["kind"] == "crack":
        _, _, p0, direction = speckle.crack_setup(st["seed"], W, H)
        dist = speckle.crack_distance(tmpl["x"], tmpl["y"], (p0, direction))
        near = dist <= R + 2
        fb = np.stack([(q["u0"] == np.round(q["u0"])) & (q["v0"] == np.round(q["v0"])) for q in results])
        out["fallback_rate_near_crack"] = float(fb[:, near].mean())
        out["fallback_rate_away_from_crack"] = float(fb[:, ~near].mean())
        out["near_crack"] = f"POIs within r + 2 = {R + 2} px of the crack line ({int(near.sum())} of {n})"
    eng.close()
    return out


def write_pgm16(path, img, maxval):
    h, w = img.shape
    Path(path).write_bytes(f"P5\n{w} {h}\n{maxval}\n".encode() + img.astype(">u2").tobytes())


def measure_cli(st, ref, frames):
    """The pipeline's process surface on a stream: opencorr_cli_gb300 --multi-frame over the
    window written as 12-bit PGMs (decode thread, staged uploads, solve, raw records, manifest,
    XXH3-128 ledger of inputs and outputs).  Steady-state frames/s from runs over all n frames
    and over the first 4 (best of three each), so process start, CUDA context, engine creation
    and reference prep cancel: (n - 4) / (wall(n) - wall(4)).  Outputs go to a tmpfs
    directory (/dev/shm: the command line's own cost) and to the temporary directory on disk,
    where the end-of-run durability barrier (directory fsync) also flushes every payload."""
    import tempfile
    cli = ROOT / "fasticgn_gb300" / "opencorr_cli_gb300"
    if not cli.exists():
        return {"unavailable": "opencorr_cli_gb300 is not built"}
    out = {"workload": st["name"], "frames": len(frames)}
    with tempfile.TemporaryDirectory(prefix="gb300_cli_") as tmp:
        d = Path(tmp)
        write_pgm16(d / "ref.pgm", ref, 4095)
        lines = []
        for k, f in enumerate(frames):
            write_pgm16(d / f"tar_{k:04d}.pgm", f, 4095)
            lines.append(f"{d / f'tar_{k:04d}.pgm'} frame_{k:06d}.csv")
        import shutil
        shm = Path("/dev/shm")
        roomy = shm.is_dir() and os.access(shm, os.W_OK) and shutil.disk_usage(shm).free > (1 << 30)
        bases = [("tmpfs", shm)] if roomy else []
        bases.append(("disk", d))
        runs = []

        def run(base, n):
            lst = d / f"list{n}.txt"
            lst.write_text("\n".join(lines[:n]) + "\n")
            o = Path(tempfile.mkdtemp(prefix="gb300_cli_out_", dir=base))   # fresh: a complete one is only verified
            runs.append(o)
            t = time.perf_counter()
            p = subprocess.run([str(cli), "--multi-frame", "--ref", str(d / "ref.pgm"), "--tar-list", str(lst),
                                "--output-dir", str(o), str(st["radius"]), str(st["step"]),
                                "--input-depth", "12", "--output-format", "raw", "--gpu-device", "0"],
                               capture_output=True, text=True, timeout=120)
            wall = time.perf_counter() - t
            shutil.rmtree(o, ignore_errors=True)   # one run's outputs at a time
            status = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
            if p.returncode != 0 or not status:
                raise RuntimeError(f"opencorr_cli_gb300 failed: {p.stderr[-400:]}")
            return wall, json.loads(status[-1])

        n, m = len(frames), 4
        try:
            run(d, m)                              # warm the page cache and the driver
            for label, base in bases:
                wm = min(run(base, m)[0] for _ in range(3))
                walls = [run(base, n) for _ in range(3)]
                wn = min(w for w, _ in walls)
                out[f"frames_per_s_{label}"] = (n - m) / (wn - wm)
                out[f"wall_s_{label}"] = {"all": wn, "first4": wm}
                out["frames_processed"] = walls[-1][1]["frames_processed"]
                out["skip_fftcc_frames"] = walls[-1][1]["totals"]["skip_fftcc_frames"]
        finally:
            for o in runs:
                shutil.rmtree(o, ignore_errors=True)
    out["timing"] = ("host wall clock of the process, best of 3; steady state = (frames - 4) / (wall(all) - "
                     "wall(first 4)); PGM decode, upload, solve, raw records + manifest + XXH3-128 ledger; tmpfs: "
                     "outputs in /dev/shm, disk: outputs on the temporary directory, whose end-of-run directory "
                     "fsync flushes every payload")
    return out


def measure_config1(dic, torch, dev):
    """The reference's CPU-runnable case: 512x512 u8, translation (2.37, -1.61) + strain 1e-3,
    noise 1 DN, r 15, step 10.  Host API per pair (upload, FFTCC + IC-GN, download), timed on
    the host clock; CPU oracle on the whole queue for the same pair."""
    from fasticgn_gb300 import speckle
    from oracle import oracle as O
    pr = speckle.pair_affine(seed=1, width=512, height=512)
    q0 = dic.grid_queue(512, 512, 15, 10)
    eng = dic.Engine(15, 15, WORKLOAD["conv"], WORKLOAD["max_iter"], device=dev.index)
    q = q0.copy()
    for _ in range(3):
        q = q0.copy()
        eng.set_ref(pr.ref)
        eng.set_tar(pr.tar)
        eng.process_pair(q)
    torch.cuda.synchronize()
    t = []
    for _ in range(20):
        q = q0.copy()
        t0 = time.perf_counter()
        eng.set_ref(pr.ref)
        eng.set_tar(pr.tar)
        eng.process_pair(q)
        t.append(time.perf_counter() - t0)
    eng.close()
    pois = O.grid_pois(512, 512, 15, 10)
    threads = O.default_threads()
    c0 = time.perf_counter()
    O.run_pair(pr.ref.astype(np.float32), pr.tar.astype(np.float32), pois, 15, threads=threads)
    cpu_s = time.perf_counter() - c0
    cz, gz = pois["r"][:, O.R_ZNCC], q["zncc"]
    both = (cz >= 0) & (gz >= 0)
    du = np.abs(pois["p"][both, O.P_U] - q["u"][both])
    dv = np.abs(pois["p"][both, O.P_V] - q["v"][both])
    ms = 1e3 * float(np.median(t))
    return {"workload": "pair512_affine_r15_step10", "pois": len(q0), "ms_per_pair_e2e": ms,
            "pois_per_s_e2e": len(q0) / (ms * 1e-3), "cpu_oracle_ms": 1e3 * cpu_s, "cpu_cores": threads,
            "parity_vs_cpu": {"median_du": float(np.median(du)), "median_dv": float(np.median(dv)),
                              "p99_du": float(np.quantile(du, .99)), "max_du": float(du.max()),
                              "max_dv": float(dv.max()),
                              "flags_agree": float(np.mean((cz >= 0) == (gz >= 0)))},
            "timing": "host clock, median of 20 pairs: set_ref + set_tar + process_pair (upload, prep, FFTCC, "
                      "IC-GN, download); the CPU oracle on the whole queue, all host threads"}


# ------------------------------------------------------------------------------ ranks
# One process per GPU (torchrun); each rank solves its own pair, so the work per rank is
# fixed (weak scaling) and no collective touches the data path: the ranks only meet at the
# barriers around the timed region and in the max-over-ranks of the timings.

def rank_info():
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(x: float, world: int, device) -> float:
    """The largest per-rank value (the whole job is as slow as its slowest rank)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, units_per_rank: int, ms_max: float) -> float:
    """Units of all ranks per second of the slowest rank."""
    return world * units_per_rank / (ms_max * 1e-3)


def run_ours(args):
    import torch
    import torch.distributed as dist
    import fasticgn_gb300 as dic
    from fasticgn_gb300 import _build, _lib, proposal

    world, rank, local = rank_info()
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    # host worker pools before any CUDA use; the batch and the streams are reported by rank 0
    uneven_jobs = load_uneven() if rank == 0 and not args.skip_batch else None
    streams = load_streams() if rank == 0 and not args.skip_streams else None
    torch.cuda.set_device(local)
    _build.build_lib()
    clock = ClockSampler(local).__enter__()     # sampled for the whole run; summaries keep timed windows

    ref, tar = load_pair()
    W, H, R = WORKLOAD["width"], WORKLOAD["height"], WORKLOAD["radius"]
    tmpl = grid()
    P = len(tmpl)
    dev = torch.device("cuda", local)
    eng = dic.Engine(R, R, WORKLOAD["conv"], WORKLOAD["max_iter"], device=local)
    eng.set_autotune(True)          # launch shapes tuned on the first (warm-up) step
    net = None
    modes = ["fftcc"]
    if proposal.WEIGHTS.exists():
        net = proposal.ProposalNet.load(device=local)
        eng.set_proposal(net)
        modes.append("learned")
    headline = args.seed if args.seed in modes else modes[-1]
    stream = torch.cuda.ExternalStream(eng.stream, device=dev)
    ref_d = torch.from_numpy(ref).to(dev)
    tar_d = torch.from_numpy(tar).to(dev)
    tmpl_d = torch.from_numpy(tmpl.view(np.uint8).copy()).to(dev)
    work_d = torch.empty_like(tmpl_d)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    flag_of = {"fftcc": _lib.DIC_RUN_FFTCC | _lib.DIC_RUN_ICGN | _lib.DIC_RUN_PREPARE,
               "learned": _lib.DIC_RUN_LEARNED | _lib.DIC_RUN_PREPARE}

    def device_step(mode):
        with torch.cuda.stream(stream):
            work_d.copy_(tmpl_d)
        eng.set_ref_device(ref_d.data_ptr(), W, H, W, _lib.DIC_U8)
        eng.set_tar_device(tar_d.data_ptr(), W, H, W, _lib.DIC_U8)
        eng.run_device(work_d.data_ptr(), P, flag_of[mode])

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def rank_max(x):
        return max_over_ranks(x, world, dev)

    kernel_keys = ("ms_prepare_ref", "ms_poi_prepare", "ms_prepare_tar", "ms_fftcc", "ms_proposal", "ms_icgn")
    res = {}
    for mode in modes:
        for _ in range(args.warmup):
            device_step(mode)
        barrier()
        launches0 = eng.stats()["kernel_launches"]
        times, kern, iters = [], {k: [] for k in kernel_keys}, []
        with clock.window(mode):
            for _ in range(args.steps):
                with torch.cuda.stream(stream):
                    flush.random_(0, 255)           # untimed L2 flush
                    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    s.record(stream)
                device_step(mode)
                with torch.cuda.stream(stream):
                    e.record(stream)
                e.synchronize()
                times.append(s.elapsed_time(e))
                st = eng.stats()
                for k in kern:
                    kern[k].append(st[k])
                iters.append(st["icgn_iterations"])
            barrier()
        ms = rank_max(float(np.sum(times)) / args.steps)
        res[mode] = {"ms_per_step": ms, "value": whole_job_rate(world, P, ms),
                     "launches_per_step": (eng.stats()["kernel_launches"] - launches0) / args.steps,
                     "kernels_ms": {k: float(np.mean(v)) for k, v in kern.items()},
                     "icgn_iterations": float(np.mean(iters)),
                     "result": work_d.cpu().numpy().view(dic.POI_DTYPE).copy()}

    # ---- what any seed can buy: IC-GN alone from seeds at a known distance from the converged
    # FFTCC-path solution (0 = the solution itself, which IC-GN confirms in one iteration),
    # on the same resident pair and layout.  The fixed part of a step (reference prep,
    # per-POI prep, target table) does not depend on the seed.
    # ---- the same FFTCC-seeded step with IC-GN sampling the B-spline coefficient table
    # (DIC_SAMPLE_TABLE, k_icgn_persistent) instead of staged pixels: the previous form,
    # timed the same way for the comparison and its L2 gather roofline
    table_form = None
    if "fftcc" in res:
        eng.set_sampling(_lib.DIC_SAMPLE_TABLE)
        for _ in range(args.warmup):
            device_step("fftcc")
        barrier()
        times, icgn, its = [], [], []
        for _ in range(max(3, args.steps // 4)):
            with torch.cuda.stream(stream):
                flush.random_(0, 255)
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.record(stream)
            device_step("fftcc")
            with torch.cuda.stream(stream):
                e.record(stream)
            e.synchronize()
            times.append(s.elapsed_time(e))
            st = eng.stats()
            icgn.append(st["ms_icgn"])
            its.append(st["icgn_iterations"])
        same = np.array_equal(work_d.cpu().numpy().view(dic.POI_DTYPE)["zncc"] < 0, res["fftcc"]["result"]["zncc"] < 0)
        table_form = {"ms_per_step": float(np.mean(times)), "value": whole_job_rate(world, P, float(np.mean(times))),
                      "ms_icgn": float(np.mean(icgn)), "icgn_iterations": float(np.mean(its)),
                      "flags_equal_to_pixel_form": bool(same), "tuning": eng.tuning()["icgn_column"]}
        eng.set_sampling(_lib.DIC_SAMPLE_PIXELS)

    seed_floor = None
    if "fftcc" in res:
        base = res["fftcc"]["result"]
        ok = base["zncc"] >= 0
        rng = np.random.default_rng(0)
        seed_floor = {"offsets_px": {}}
        for off in (0.0, 0.05, 0.2, 0.5):
            q = tmpl.copy()
            for f in ("u", "ux", "uy", "v", "vx", "vy"):
                q[f] = np.where(ok, base[f], 0.0)
            if off:
                ang = rng.uniform(0, 2 * np.pi, P)
                q["u"] += np.where(ok, off * np.cos(ang), 0.0).astype(np.float32)
                q["v"] += np.where(ok, off * np.sin(ang), 0.0).astype(np.float32)
            qd = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
            ms, its = [], []
            for k in range(args.warmup + args.steps):
                with torch.cuda.stream(stream):
                    work_d.copy_(qd)
                    flush.random_(0, 255)
                eng.run_device(work_d.data_ptr(), P, _lib.DIC_RUN_ICGN)
                st = eng.stats()
                if k >= args.warmup:
                    ms.append(st["ms_icgn"])
                    its.append(st["icgn_iterations"] / P)
            seed_floor["offsets_px"][str(off)] = {"icgn_ms": float(np.mean(ms)), "iterations_per_poi": float(np.mean(its))}
        fixed = sum(res["fftcc"]["kernels_ms"][k] for k in ("ms_prepare_ref", "ms_poi_prepare", "ms_prepare_tar"))
        seed_floor["fixed_ms"] = fixed
        seed_floor["fftcc_step_ms"] = res["fftcc"]["ms_per_step"]
        # ceiling of learned / FFTCC-seeded throughput for a proposal that costs nothing and
        # lands at that distance from the solution
        for off, v in seed_floor["offsets_px"].items():
            v["ceiling_vs_fftcc_at_zero_proposal_cost"] = res["fftcc"]["ms_per_step"] / (fixed + v["icgn_ms"])
        seed_floor["note"] = ("IC-GN from the converged FFTCC-path solution moved by the given distance in a random "
                              "direction (valid POIs); the ceiling adds no proposal time")

    # ---- e2e through the host C ABI (pinned host buffers), headline mode
    ref_h = torch.from_numpy(ref).pin_memory()
    tar_h = torch.from_numpy(tar).pin_memory()
    q_h = torch.from_numpy(tmpl.view(np.uint8).copy()).pin_memory()
    q_np = q_h.numpy().view(dic.POI_DTYPE)
    tmpl_bytes = tmpl.view(np.uint8)

    def e2e_step():
        eng.set_ref(ref_h.numpy())
        eng.set_tar(tar_h.numpy())
        if headline == "learned":
            eng.process_pair_learned(q_np)
        else:
            eng.process_pair(q_np)

    for _ in range(max(1, args.warmup)):
        q_h.numpy()[:] = tmpl_bytes
        e2e_step()
    e2e_times = []
    gc.disable()   # no collector pause inside a timed step
    e2e_win = clock.window("e2e")
    e2e_win.__enter__()
    for _ in range(args.steps):
        q_h.numpy()[:] = tmpl_bytes          # the caller's fresh POI queue (untimed)
        with torch.cuda.stream(stream):
            flush.random_(0, 255)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        e2e_step()
        e.record(stream)
        e.synchronize()
        e2e_times.append(s.elapsed_time(e))
    e2e_win.__exit__(None, None, None)
    gc.enable()
    e2e_ms = rank_max(float(np.mean(e2e_times)))
    assert q_np.tobytes() == res[headline]["result"].tobytes(), "host and device entry points disagree"

    uneven = None
    if uneven_jobs is not None:
        uneven = measure_uneven(dic, torch, dev, flush, uneven_jobs, max(5, min(args.steps, 20)), args.warmup, clock)
    config1 = measure_config1(dic, torch, dev) if rank == 0 else None
    stream_lines = None
    cli_line = None
    if streams is not None:
        stream_lines = {st["name"]: measure_stream(dic, torch, dev, st, *streams[st["name"]], net, flush, clock)
                        for st in STREAMS}
        if rank == 0:
            st0 = STREAMS[0]
            cli_line = measure_cli(st0, *streams[st0["name"]])

    peaks = measure_read_peak(torch, dev) if rank == 0 else None
    clock.__exit__(None, None, None)
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant kernel, IC-GN under pixel sampling (k_icgn_px).  Each warped
    # sample reads its 4 x 4 pixel support (16 x 4 B) from the POI's window in shared memory;
    # an iteration on the pixel lattice (the first one from an integer FFTCC seed) reads one
    # pixel per sample.  The reference texel (16 B) per sample per iteration comes through
    # L1/L2, and each POI's window (bx x by floats) is staged once from L2 by TMA.  The bound
    # is the shared-memory load bandwidth, measured in this run by dic_smem_probe; ncu shows
    # the kernel limited by instruction issue below it (issue_active_pct_ncu).
    N = (2 * R + 1) ** 2
    H0 = res[headline]
    icgn_ms = H0["kernels_ms"]["ms_icgn"]
    iters = H0["icgn_iterations"]
    lattice_iters = float(np.sum(H0["result"]["iteration"] >= 1)) if headline == "fftcc" else 0.0
    smem_bytes = N * (64.0 * (iters - lattice_iters) + 4.0 * lattice_iters)
    wx, wy = ((2 * R + 1 + 3 + 2 + 1 + 3) + 3) // 4 * 4, 2 * R + 1 + 3 + 2 + 1
    l2_bytes = 16.0 * N * iters + P * (4.0 * wx * wy + 224 + 2 * 56)
    achieved = smem_bytes / (icgn_ms * 1e-3) / 1e9
    prof = profiled("k_icgn_px")
    traffic = prof.get("dram_bytes_per_launch")
    hbm_peak, hbm_kind = measured_peak_hbm()
    roofline = {"kernel": "k_icgn_px", "bound": "smem", "achieved": achieved, "peak": peaks["smem"]["gbs"],
                "unit": "GB/s", "frac": achieved / peaks["smem"]["gbs"],
                "peak_source": ("measured in this run: dic_smem_probe, conflict-free 32-float warp loads from "
                                "shared memory, 8 CTAs of 256 threads per SM (of measured)"),
                "traffic": traffic, "algorithmic_bytes_per_launch": smem_bytes, "icgn_ms": icgn_ms,
                "model": "64 B of pixels per warped sample per iteration from the staged window (4 B on the "
                         "pixel lattice); per-launch counts from the step's own iteration total",
                "issue_active_pct_ncu": prof.get("issue_active_pct"),
                "limiter_ncu": prof.get("limiter"),
                "l2": {"achieved": l2_bytes / (icgn_ms * 1e-3) / 1e9, "peak": peaks["l2"]["gbs"],
                       "frac": l2_bytes / (icgn_ms * 1e-3) / 1e9 / peaks["l2"]["gbs"],
                       "model": "16 B reference texel per sample per iteration + one pixel window, the "
                                "record and the queue per POI", "busy_pct_ncu": prof.get("lts_throughput_pct")},
                "hbm": {"achieved": (traffic / (icgn_ms * 1e-3) / 1e9) if traffic else None, "peak": hbm_peak,
                        "frac": (traffic / (icgn_ms * 1e-3) / 1e9 / hbm_peak) if traffic else None,
                        "peak_source": hbm_kind, "note": "DRAM bytes per launch (ncu) over the IC-GN time"},
                "read_probe": peaks, "profile_source": prof.get("source")}
    if table_form is not None:
        # the table form's gathers: 64 B of coefficients per sample per iteration (4 B on the
        # lattice plane) + 16 B reference texel, served by L2
        t_bytes = N * (64.0 * (iters - lattice_iters) + 4.0 * lattice_iters) + 16.0 * N * iters + P * (224 + 2 * 56)
        t_ach = t_bytes / (table_form["ms_icgn"] * 1e-3) / 1e9
        table_form["l2_roofline"] = {"kernel": "k_icgn_persistent", "bound": "l2", "achieved": t_ach,
                                     "peak": peaks["l2"]["gbs"], "frac": t_ach / peaks["l2"]["gbs"],
                                     "model": "64 B coefficient texel per sample per iteration (4 B lattice) + "
                                              "16 B reference texel + record per POI"}
        roofline["table_form"] = table_form

    # ---- the other hot kernels against their own bounds (FLOP models per POI)
    M = 2 * R
    fftcc_flop = 2 * (2.5 * M * M * np.log2(M * M)) + 6 * M * (M // 2 + 1) + 4 * M * M
    fp32_peak = peaks["fp32"]["tflops"]             # measured in this run by dic_fma_probe
    try:
        bf16_peak = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"])
        bf16_src = "measured"
    except (OSError, KeyError, ValueError):
        bf16_peak, bf16_src = 1900.0, "fallback"
    other = {"k_fftcc": {"bound": "fp32", "flop_per_poi": fftcc_flop,
                         "achieved": fftcc_flop * P / (H0["kernels_ms"]["ms_fftcc"] * 1e-3) / 1e12,
                         "peak": fp32_peak, "unit": "TFLOP/s",
                         "peak_source": "measured in this run: dic_fma_probe, 8 independent FMA chains per thread"}}
    if "learned" in res:
        cnn_flop = 2 * (256 * 32 * 18 + 64 * 32 * 288 + 16 * 32 * 288 + 4 * 32 * 288 + 128 * 256 + 256 * 6)
        other["k_proposal_fused"] = {"bound": "tensor", "flop_per_poi": cnn_flop,
                                     "achieved": cnn_flop * P / (res["learned"]["kernels_ms"]["ms_proposal"] * 1e-3) / 1e12,
                                     "peak": bf16_peak, "unit": "TFLOP/s", "peak_source": bf16_src}
    for v in other.values():
        v["frac"] = v["achieved"] / v["peak"]

    # ---- CPU baseline on the whole queue, and parity of each GPU mode against its results
    from oracle import oracle as O
    threads = O.default_threads()
    cpu_value, cpu_detail, cpu_result = cpu_pair_time(ref, tar, threads)
    seed_modes = {}
    for mode, r in res.items():
        ok = r["result"]["zncc"] >= 0
        its = r["result"]["iteration"][ok].astype(np.int64)
        hist = np.bincount(its, minlength=WORKLOAD["max_iter"] + 1)
        seed_modes[mode] = {"value": r["value"], "ms_per_step": r["ms_per_step"], "kernels_ms": r["kernels_ms"],
                            "icgn_iterations_per_poi": r["icgn_iterations"] / P, "valid_ratio": float(ok.mean()),
                            "iterations_histogram": {str(k): int(c) for k, c in enumerate(hist) if c},
                            "fftcc_fallback_ratio": (float(np.mean((r["result"]["u0"] == np.round(r["result"]["u0"])) &
                                                                   (r["result"]["v0"] == np.round(r["result"]["v0"]))))
                                                     if mode == "learned" else None),
                            "kernel_launches_per_step": r["launches_per_step"],
                            "parity_vs_cpu": parity_vs_cpu(r["result"], cpu_result)}
    h2d = ref.nbytes + tar.nbytes + tmpl.nbytes
    cfg = config_block()
    cfg["seed_method"] = {"fftcc": "FFTCC", "learned": "learned proposal CNN (FFTCC fallback)"}[headline]
    line = {
        "metric": "POIs/s", "value": H0["value"], "unit": "POI/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": H0["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (IC-GN, FFTCC); bf16 tensor-core with f32 accumulation (proposal CNN)",
        "data": "synthetic", "config": cfg,
        "frames_per_s": world * 1e3 / H0["ms_per_step"],
        "e2e": {"value": whole_job_rate(world, P, e2e_ms), "unit": "POI/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(tmpl.nbytes)},
        "roofline": roofline,
        "roofline_other_kernels": other,
        "cpu_baseline": {"value": cpu_value, "unit": "POI/s", "cores": threads, "kind": "port",
                         "sample": CPU_SAMPLE, "detail": cpu_detail},
        "clocks": clock.summary(),
        "clocks_headline": clock.summary([headline]),
        "gpu_launches": int(round(H0["launches_per_step"] * args.steps)),
        "icgn_launch_shape": eng.tuning()["icgn_column_px"],
        "seed_modes": seed_modes,
        "learned_vs_fftcc": (seed_modes["learned"]["value"] / seed_modes["fftcc"]["value"]) if "learned" in seed_modes else None,
        "seed_floor": seed_floor,
        "parity_vs_cpu": seed_modes[headline]["parity_vs_cpu"],
        "config1_pair512": config1,
        "uneven_batch": uneven,
        "streams": stream_lines,
        "cli_stream": cli_line,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def profile_pair(radius):
    """One small, fixed launch sequence for an ncu capture: the bench's 2048x2048 pair at the
    given subset radius, step 4, solved twice on one engine with the untuned launch shapes
    (about 0.2 GB of planes and records on the device)."""
    import fasticgn_gb300 as dic
    ref, tar = load_pair()
    h, w = ref.shape
    q0 = dic.grid_queue(w, h, radius, 4)
    e = dic.Engine(radius, radius, WORKLOAD["conv"], WORKLOAD["max_iter"])
    e.set_autotune(False)
    e.set_timing(True)
    for _ in range(2):
        q = q0.copy()
        e.set_ref(ref)
        e.set_tar(tar)
        e.process_pair(q)
    st = e.stats()
    print(json.dumps({"radius": radius, "pois": len(q0), **{k: st[k] for k in st if k.startswith("ms_")}}))
    e.close()


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--skip-batch", action="store_true", help="do not measure the uneven batch")
    ap.add_argument("--skip-streams", action="store_true", help="do not measure the frame streams")
    ap.add_argument("--seed", choices=["fftcc", "learned"], default="fftcc",
                    help="seed method of the headline value (both are measured when the proposal weights exist)")
    ap.add_argument("--profile-pair", type=int, default=0, metavar="R",
                    help="profiling driver: solve the 2048x2048 pair at subset radius R (step 4, untuned default "
                         "launch shapes) twice and print the second solve's kernel times; nothing else runs")
    args = ap.parse_args()
    if args.profile_pair:
        profile_pair(args.profile_pair)
        return
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

"""Proposal network: learned seeds for IC-GN (no counterpart in the reference).

A small CNN (csrc/dic_cnn.cuh) maps the 31x31 reference and target windows at a POI to
(u, v, ux, uy, vx, vy).  It is trained on pairs the method generates itself: synthetic
speckle warped by smooth random fields, labelled by this engine's converged FFTCC-seeded
IC-GN.  Training runs on the GPU through dic_cnn_train_step (BF16 tensor-core forward and
backward, FP32 accumulation, Adam on FP32 master weights).  torch is used only to hold
device buffers.

    net = ProposalNet.load()                 # weights/proposal_r15.npz
    eng = Engine(15); eng.set_proposal(net)  # then eng.process_pair_learned(queue)
"""
from __future__ import annotations

import ctypes
import time
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import POI_DTYPE

WEIGHTS = Path(__file__).resolve().parent / "weights" / "proposal_r15.npz"
ACCEPT_ZNCC = 0.9


def _torch():
    import torch
    return torch


class ProposalNet:
    def __init__(self, device: int = 0, params: np.ndarray | None = None):
        self._L = _lib.load()
        h = ctypes.c_void_p()
        rc = self._L.dic_cnn_create(int(device), ctypes.byref(h))
        if rc != _lib.DIC_OK:
            raise _lib.DicError(rc, "dic_cnn_create failed (is a CUDA device available?)")
        self._h = h
        self.device = device
        self.count = int(self._L.dic_cnn_param_count())
        if params is not None:
            self.set_params(params)

    def close(self):
        if getattr(self, "_h", None):
            self._L.dic_cnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _call(self, rc):
        if rc != _lib.DIC_OK:
            msg = self._L.dic_cnn_last_error(self._h)
            raise _lib.DicError(rc, msg.decode() if msg else "")

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.shape != (self.count,):
            raise ValueError(f"expected {self.count} parameters")
        self._call(self._L.dic_cnn_set_params(self._h, p.ctypes.data, self.count))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.count, dtype=np.float32)
        self._call(self._L.dic_cnn_get_params(self._h, p.ctypes.data, self.count))
        return p

    def save(self, path: Path = WEIGHTS, **meta):
        path = Path(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        np.savez_compressed(path, params=self.get_params(), **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path: Path = WEIGHTS, device: int = 0) -> "ProposalNet":
        d = np.load(path)
        return cls(device, d["params"])

    # --- device-tensor entry points (torch tensors on the network's device)
    def inputs(self, ref_f32, tar_f32, pois_dev, n: int):
        """BF16 [n, 31, 31, 2] windows for the POIs in pois_dev (a uint8 tensor of dic_poi records)."""
        torch = _torch()
        h, w = ref_f32.shape
        x0 = torch.empty((n, 31, 31, 2), dtype=torch.bfloat16, device=ref_f32.device)
        self._call(self._L.dic_cnn_input(self._h, ref_f32.data_ptr(), tar_f32.data_ptr(), w, h, pois_dev.data_ptr(),
                                         n, x0.data_ptr()))
        return x0

    def seed(self, ref_f32, tar_f32, pois_dev, n: int):
        """Fused inference: proposal seeds written into the dic_poi records of pois_dev."""
        h, w = ref_f32.shape
        _torch().cuda.synchronize()
        self._call(self._L.dic_cnn_seed(self._h, ref_f32.data_ptr(), tar_f32.data_ptr(), w, h, pois_dev.data_ptr(), n))

    def forward(self, x0):
        torch = _torch()
        out = torch.empty((x0.shape[0], 8), dtype=torch.float32, device=x0.device)
        torch.cuda.synchronize()
        self._call(self._L.dic_cnn_forward(self._h, x0.data_ptr(), x0.shape[0], out.data_ptr()))
        return out

    def gradient(self, x0, target):
        torch = _torch()
        g = torch.empty(self.count, dtype=torch.float32, device=x0.device)
        loss = ctypes.c_float()
        torch.cuda.synchronize()
        self._call(self._L.dic_cnn_gradient(self._h, x0.data_ptr(), target.data_ptr(), x0.shape[0], g.data_ptr(),
                                            ctypes.byref(loss)))
        return loss.value, g

    def train_step(self, x0, target, lr: float) -> float:
        loss = ctypes.c_float()
        self._call(self._L.dic_cnn_train_step(self._h, x0.data_ptr(), target.data_ptr(), x0.shape[0], float(lr),
                                              ctypes.byref(loss)))
        return loss.value


def init_params(seed: int = 0) -> np.ndarray:
    """He initialisation in the network's parameter layout (csrc/dic_cnn.cuh ParamLayout)."""
    rng = np.random.default_rng(seed)
    sizes = [("w", 32 * 9 * 2, 18), ("b", 32, 0), ("w", 32 * 9 * 32, 288), ("b", 32, 0), ("w", 32 * 9 * 32, 288),
             ("b", 32, 0), ("w", 32 * 9 * 32, 288), ("b", 32, 0), ("w", 256 * 128, 128), ("b", 256, 0),
             ("w", 6 * 256, 256), ("b", 6, 0)]
    parts = []
    for i, (kind, n, fan) in enumerate(sizes):
        if kind == "b":
            parts.append(np.zeros(n, np.float32))
        else:
            gain = 0.5 if i == 10 else 1.0
            parts.append(rng.normal(0.0, gain * np.sqrt(2.0 / fan), n).astype(np.float32))
    return np.concatenate(parts)


def training_set(pairs, radius: int = 15, step: int = 4, device: int = 0, accept: float = ACCEPT_ZNCC,
                 max_samples: int | None = None, rng=None):
    """Inputs and labels from synthetic pairs: each pair is solved by this engine's FFTCC-seeded
    IC-GN and every POI that converged with ZNCC >= accept becomes one sample.

    pairs: iterable of (ref u8, tar u8).  Returns (x0 bf16 [N,31,31,2], targets f32 [N,6]) on
    the device."""
    torch = _torch()
    from .engine import Engine, grid_queue
    net = ProposalNet(device)
    xs, ts = [], []
    dev = torch.device("cuda", device)
    for ref, tar in pairs:
        h, w = ref.shape
        q = grid_queue(w, h, radius, step)
        with Engine(radius, radius, 0.001, 10, device=device) as e:
            e.set_ref(ref)
            e.set_tar(tar)
            e.process_pair(q)
        ok = (q["zncc"] >= accept) & (q["iteration"] < 10)
        q = np.ascontiguousarray(q[ok])
        if rng is not None and max_samples is not None and len(q) > max_samples:
            q = np.ascontiguousarray(q[np.sort(rng.choice(len(q), max_samples, replace=False))])
        qd = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
        rf = torch.from_numpy(ref.astype(np.float32)).to(dev)
        tf = torch.from_numpy(tar.astype(np.float32)).to(dev)
        xs.append(net.inputs(rf, tf, qd, len(q)))
        t = np.stack([q["u"], q["v"], q["ux"], q["uy"], q["vx"], q["vy"]], axis=1).astype(np.float32)
        ts.append(torch.from_numpy(t).to(dev))
    net.close()
    return torch.cat(xs), torch.cat(ts)


def train(net: ProposalNet, x0, targets, steps: int, batch: int = 2048, lr: float = 2e-3, seed: int = 0,
          log_every: int = 0):
    """Adam with a cosine learning-rate decay over random mini-batches; returns the loss history."""
    torch = _torch()
    g = torch.Generator(device=x0.device)
    g.manual_seed(seed)
    n = x0.shape[0]
    losses = []
    t0 = time.time()
    for s in range(steps):
        idx = torch.randint(0, n, (batch,), device=x0.device, generator=g)
        xb = x0.index_select(0, idx).contiguous()
        tb = targets.index_select(0, idx).contiguous()
        torch.cuda.synchronize()
        rate = lr * 0.5 * (1.0 + np.cos(np.pi * s / steps))
        losses.append(net.train_step(xb, tb, max(rate, lr * 0.01)))
        if log_every and (s % log_every == 0 or s == steps - 1):
            print(f"step {s:5d} loss {losses[-1]:.5f} ({time.time() - t0:.1f} s)", flush=True)
    return losses


def synthetic_pairs(count: int, seed: int = 100, size: int = 1024, max_disp: float = 12.0, max_strain: float = 0.02):
    """Pairs from the learned-seed workload's field distribution (smooth Gaussian-bump fields)."""
    from . import speckle
    for k in range(count):
        pr = speckle.pair_bumps(seed=seed + k, width=size, height=size, max_disp=max_disp, max_strain=max_strain)
        yield pr.ref, pr.tar


def main():
    import argparse
    ap = argparse.ArgumentParser(description="Train the proposal network on method-generated pairs")
    ap.add_argument("--pairs", type=int, default=8)
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--out", type=Path, default=WEIGHTS)
    args = ap.parse_args()
    t = time.time()
    x0, tg = training_set(synthetic_pairs(args.pairs, size=args.size))
    print(f"{x0.shape[0]} samples in {time.time() - t:.1f} s", flush=True)
    net = ProposalNet(0, init_params(0))
    losses = train(net, x0, tg, args.steps, args.batch, args.lr, log_every=250)
    net.save(args.out, samples=x0.shape[0], steps=args.steps, batch=args.batch, lr=args.lr,
             final_loss=float(np.mean(losses[-50:])), pairs=args.pairs, size=args.size)
    print(f"saved {args.out}")


if __name__ == "__main__":
    main()

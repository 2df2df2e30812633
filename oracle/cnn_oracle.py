"""TEST INFRASTRUCTURE: float64 CPU forward/backward of the proposal network.

Restates fasticgn_gb300/csrc/dic_cnn.cuh in numpy: the same parameter layout, NHWC
activations, 3x3 stride-2 pad-1 convolutions, ReLU, the 128-256-6 MLP and the MSE loss on
(u, v, 100 ux, 100 uy, 100 vx, 100 vy).  With ``bf16=True`` it rounds to BF16 exactly where
the GPU stores BF16 (working weights, the input, every ReLU output, dL/dout and every
masked back-propagated gradient) and accumulates in float64, so GPU-vs-oracle differences
come only from the GPU's FP32 accumulation order.  With ``bf16=False`` it is the plain
float64 network, used for finite differences and against torch autograd.
"""
from __future__ import annotations

import numpy as np

WIN, CH, HID, OUT = 31, 32, 256, 6
SIDES = [31, 16, 8, 4, 2]
SCALE = np.array([1.0, 1.0, 100.0, 100.0, 100.0, 100.0])


def _layout():
    off, lay = 0, {}
    for name, size in (("w1", 32 * 9 * 2), ("b1", 32), ("w2", 32 * 9 * 32), ("b2", 32), ("w3", 32 * 9 * 32),
                       ("b3", 32), ("w4", 32 * 9 * 32), ("b4", 32), ("w5", HID * 128), ("b5", HID),
                       ("w6", OUT * HID), ("b6", OUT)):
        lay[name] = (off, size)
        off += size
    return lay, off


LAYOUT, PARAM_COUNT = _layout()
assert PARAM_COUNT == 62918


def bf16(x):
    """Round float32 values to BF16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32)
    r = ((a >> 16) & 1) + np.uint32(0x7FFF)
    return ((a + r) & np.uint32(0xFFFF0000)).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    t = {k: p[o:o + n] for k, (o, n) in LAYOUT.items()}
    return {
        "w": [t["w1"].reshape(32, 3, 3, 2), t["w2"].reshape(32, 3, 3, 32), t["w3"].reshape(32, 3, 3, 32),
              t["w4"].reshape(32, 3, 3, 32)],
        "b": [t["b1"], t["b2"], t["b3"], t["b4"]],
        "w5": t["w5"].reshape(HID, 128), "b5": t["b5"], "w6": t["w6"].reshape(OUT, HID), "b6": t["b6"],
    }


def pack_grads(g):
    out = np.zeros(PARAM_COUNT)
    parts = {"w1": g["w"][0], "b1": g["b"][0], "w2": g["w"][1], "b2": g["b"][1], "w3": g["w"][2], "b3": g["b"][2],
             "w4": g["w"][3], "b4": g["b"][3], "w5": g["w5"], "b5": g["b5"], "w6": g["w6"], "b6": g["b6"]}
    for k, (o, n) in LAYOUT.items():
        out[o:o + n] = np.asarray(parts[k]).ravel()
    return out


def im2col(x, so):
    """x: [n, s, s, c] -> [n, so, so, 9*c] with k = (ky, kx, c), stride 2, pad 1."""
    n, s, _, c = x.shape
    xp = np.zeros((n, s + 2, s + 2, c))
    xp[:, 1:s + 1, 1:s + 1] = x
    cols = np.zeros((n, so, so, 9, c))
    for ky in range(3):
        for kx in range(3):
            cols[:, :, :, ky * 3 + kx] = xp[:, ky:ky + 2 * so:2, kx:kx + 2 * so:2][:, :so, :so]
    return cols.reshape(n, so, so, 9 * c)


def col2im(dcols, s, c):
    """Adjoint of im2col: dcols [n, so, so, 9*c] -> dx [n, s, s, c]."""
    n, so = dcols.shape[0], dcols.shape[1]
    d = dcols.reshape(n, so, so, 9, c)
    dxp = np.zeros((n, s + 2 + 2, s + 2 + 2, c))
    for ky in range(3):
        for kx in range(3):
            dxp[:, ky:ky + 2 * so:2, kx:kx + 2 * so:2][:, :so, :so] += d[:, :, :, ky * 3 + kx]
    return dxp[:, 1:s + 1, 1:s + 1]


def forward(params, x0, bf=True):
    q = bf16 if bf else (lambda v: np.asarray(v, dtype=np.float64))
    P = unpack(params)
    acts = [q(x0)]
    for l in range(4):
        so, ci = SIDES[l + 1], (2 if l == 0 else 32)
        cols = im2col(acts[-1], so)
        w = q(P["w"][l].reshape(32, 9 * ci))
        z = cols @ w.T + P["b"][l]
        acts.append(q(np.maximum(z, 0.0)))
    n = x0.shape[0]
    a4 = acts[4].reshape(n, 128)
    a5 = q(np.maximum(a4 @ q(P["w5"]).T + P["b5"], 0.0))
    out = a5 @ q(P["w6"]).T + P["b6"]
    return out, {"acts": acts, "a4": a4, "a5": a5}


def loss_and_grad(params, x0, target, bf=True):
    q = bf16 if bf else (lambda v: np.asarray(v, dtype=np.float64))
    P = unpack(params)
    out, c = forward(params, x0, bf)
    n = x0.shape[0]
    t = np.asarray(target, dtype=np.float64) * SCALE
    d = out - t
    loss = float(np.sum(d * d) / (n * OUT))
    dout = q(np.asarray(d * (2.0 / (n * OUT)), dtype=np.float32)) if bf else d * (2.0 / (n * OUT))
    g = {"w": [None] * 4, "b": [None] * 4}
    g["w6"] = dout.T @ c["a5"]
    g["b6"] = dout.sum(0)
    d5 = q((dout @ q(P["w6"])) * (c["a5"] > 0))
    g["w5"] = d5.T @ c["a4"]
    g["b5"] = d5.sum(0)
    dz = q((d5 @ q(P["w5"])) * (c["a4"] > 0)).reshape(n, 2, 2, 32)
    acts = c["acts"]
    for l in range(3, -1, -1):
        si, so, ci = SIDES[l], SIDES[l + 1], (2 if l == 0 else 32)
        cols = im2col(acts[l], so)
        g["w"][l] = (dz.reshape(-1, 32).T @ cols.reshape(-1, 9 * ci)).reshape(32, 3, 3, ci)
        g["b"][l] = dz.reshape(-1, 32).sum(0)
        if l > 0:
            dcols = dz.reshape(-1, 32) @ q(P["w"][l].reshape(32, 9 * ci))
            dx = col2im(dcols.reshape(n, so, so, 9 * ci), si, ci)
            dz = q(dx * (acts[l] > 0))
    return loss, pack_grads(g), out


def init_params(seed=0):
    """He-style initialisation used for training from scratch."""
    rng = np.random.default_rng(seed)
    p = np.zeros(PARAM_COUNT, dtype=np.float32)
    fan = {"w1": 18, "w2": 288, "w3": 288, "w4": 288, "w5": 128, "w6": HID}
    for k, (o, n) in LAYOUT.items():
        if k.startswith("w"):
            p[o:o + n] = rng.normal(0.0, np.sqrt(2.0 / fan[k]) * (0.5 if k == "w6" else 1.0), n)
    return p

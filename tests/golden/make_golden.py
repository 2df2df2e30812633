"""Regenerate the golden fixtures in tests/golden/ from the reference's own generators.

Run in a container that has the reference checkout (it is not needed afterwards):

    python tests/golden/make_golden.py --reference /path/to/FastICGN

Fixtures (compressed .npz, a few hundred KB in all):

* s15.npz, s15_lowsnr.npz, s63.npz -- smoke/generate_subpixel_speckle.py build_sequence()
  with the motions, sizes, contrast and noise of smoke/run_subpixel_accuracy_gate.py:111-131;
  ground truth is the affine motion (truth is exact: images are rendered analytically).
  The accuracy limits of :134-144 are copied into the fixture as `limits`.
* shift.npz -- smoke/generate_synthetic_dic.py make_base(160, 128, seed 20260703) and
  whole-pixel shifted frames (dx, dy) = (i % 3, (i // 3) % 3), the CPU/GPU parity sequence
  of smoke/run_v9_cpu_gpu_parity.sh; truth u = dx, v = dy exactly.
* oob.npz -- smoke/run_oob_rejection_gate.py: make_base(320, 240, seed 20260917) and the
  same image shifted 10 px in x; the closed-form band of POIs that must be -3.
* zero_texture.npz -- smoke/run_zero_texture_gate.py: make_base(320, 160, seed 20261019)
  with three constant 40x40 blocks painted in, the unshifted copy and a 3-px shift with
  the blocks repainted.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def load_module(path: Path, name: str):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def read_pgm(path: Path) -> np.ndarray:
    data = path.read_bytes()
    parts = data.split(b"\n", 3)
    w, h = map(int, parts[1].split())
    return np.frombuffer(parts[3], dtype=np.uint8, count=w * h).reshape(h, w).copy()


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", type=Path, required=True, help="FastICGN checkout")
    args = ap.parse_args()
    smoke = args.reference / "smoke"
    sys.path.insert(0, str(smoke))
    speckle = load_module(smoke / "generate_subpixel_speckle.py", "generate_subpixel_speckle")
    synth = load_module(smoke / "generate_synthetic_dic.py", "generate_synthetic_dic")
    gate = load_module(smoke / "run_subpixel_accuracy_gate.py", "run_subpixel_accuracy_gate")
    zt = load_module(smoke / "run_zero_texture_gate.py", "run_zero_texture_gate")

    for name, case in gate.CASES.items():
        with tempfile.TemporaryDirectory() as tmp:
            root = Path(tmp)
            speckle.build_sequence(root, case["width"], case["height"], case["motions"],
                                   contrast=case["contrast"], noise_sigma=case["noise"])
            truth = json.loads((root / "truth.json").read_text())
            ref = read_pgm(root / "ref.pgm")
            tars = np.stack([read_pgm(root / f["file"]) for f in truth["frames"]])
        lim = gate.LIMITS[name]
        np.savez_compressed(
            HERE / f"{name}.npz", ref=ref, tars=tars, motions=np.array(case["motions"], dtype=np.float64),
            radius=case["radius"], grid=case["grid"], centre=np.array(truth["centre"]),
            limits=json.dumps({k: list(v) if isinstance(v, tuple) else v for k, v in lim.items()}))
        print(name, ref.shape, tars.shape)

    w, h = 160, 128
    base = synth.make_base(w, h, 20260703)
    shifts = [(i % 3, (i // 3) % 3) for i in range(6)]
    frames = [np.frombuffer(bytes(synth.shifted_image(w, h, base, dx, dy, fill=127)), dtype=np.uint8).reshape(h, w)
              for dx, dy in shifts]
    np.savez_compressed(HERE / "shift.npz", ref=np.frombuffer(bytes(base), dtype=np.uint8).reshape(h, w),
                        tars=np.stack(frames), shifts=np.array(shifts), radius=15)
    print("shift", len(frames))

    w, h = 320, 240
    base = synth.make_base(w, h, 20260917)
    tar = synth.shifted_image(w, h, base, 10, 0, fill=127)
    np.savez_compressed(HERE / "oob.npz", ref=np.frombuffer(bytes(base), dtype=np.uint8).reshape(h, w),
                        tar=np.frombuffer(bytes(tar), dtype=np.uint8).reshape(h, w), shift=10, radius=15)
    print("oob")

    w, h = 320, 160
    base = zt.paint_blocks(w, h, synth.make_base(w, h, 20261019))
    shifted = zt.paint_blocks(w, h, synth.shifted_image(w, h, base, 3, 0, fill=zt.FILL))
    np.savez_compressed(HERE / "zero_texture.npz", ref=np.frombuffer(bytes(base), dtype=np.uint8).reshape(h, w),
                        tar_shift=np.frombuffer(bytes(shifted), dtype=np.uint8).reshape(h, w), radius=7, shift=3,
                        block_side=zt.BLOCK_SIDE, block_y=zt.BLOCK_Y,
                        block_x=np.array([zt.BLOCK_X[k] for k in zt.BLOCKS]),
                        block_value=np.array([zt.BLOCKS[k] for k in zt.BLOCKS]))
    print("zero_texture")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())

"""File helpers for the command-line tests: PGM / TIFF writers and a reader of the
opencorr-gpu-raw-v1 records and manifest, restated from the documented layout
(docs/output-format.md:28-47 and :253-330 of the reference; pipeline/fasticgn_io.py:92-316
reads them the same way)."""
from __future__ import annotations

import json
import struct
import subprocess
from pathlib import Path

import numpy as np

RAW_DTYPE = np.dtype([("x", "<i4"), ("y", "<i4"), ("u", "<f4"), ("v", "<f4"), ("ux", "<f4"), ("uy", "<f4"),
                      ("vx", "<f4"), ("vy", "<f4"), ("zncc", "<f4")])
CSV_FIELD_ORDER = ("x", "y", "u", "v", "zncc", "uy", "vy", "ux", "vx")


def write_pgm(path: Path, img: np.ndarray, maxval: int | None = None, ascii_: bool = False) -> None:
    h, w = img.shape
    maxval = maxval or (255 if img.dtype == np.uint8 else 65535)
    head = f"P{'2' if ascii_ else '5'}\n# test image\n{w} {h}\n{maxval}\n".encode()
    if ascii_:
        body = "\n".join(" ".join(str(int(v)) for v in row) for row in img).encode() + b"\n"
    elif maxval > 255:
        body = img.astype(">u2").tobytes()
    else:
        body = img.astype(np.uint8).tobytes()
    Path(path).write_bytes(head + body)


def write_tiff(path: Path, img: np.ndarray, big_endian: bool = False, rows_per_strip: int = 7) -> None:
    """Baseline uncompressed grey TIFF, several strips."""
    h, w = img.shape
    bits = 8 if img.dtype == np.uint8 else 16
    e = ">" if big_endian else "<"
    data = img.astype(np.uint8 if bits == 8 else e + "u2").tobytes()
    row = w * bits // 8
    strips = [data[y * row:min(h, y + rows_per_strip) * row] for y in range(0, h, rows_per_strip)]
    n_strips = len(strips)
    header = (b"MM" if big_endian else b"II") + struct.pack(e + "HI", 42, 8)
    entries = 9
    ifd_size = 2 + 12 * entries + 4
    offsets_at = 8 + ifd_size
    counts_at = offsets_at + 4 * n_strips
    data_at = counts_at + 4 * n_strips
    offs, pos = [], data_at
    for s in strips:
        offs.append(pos)
        pos += len(s)

    def entry(tag, typ, count, value):
        if typ == 3 and count == 1:
            return struct.pack(e + "HHIHH", tag, typ, count, value, 0)
        return struct.pack(e + "HHII", tag, typ, count, value)

    ifd = struct.pack(e + "H", entries)
    ifd += entry(256, 4, 1, w) + entry(257, 4, 1, h) + entry(258, 3, 1, bits) + entry(259, 3, 1, 1)
    ifd += entry(262, 3, 1, 1)
    ifd += entry(273, 4, n_strips, offsets_at if n_strips > 1 else offs[0])
    ifd += entry(277, 3, 1, 1) + entry(278, 4, 1, rows_per_strip)
    ifd += entry(279, 4, n_strips, counts_at if n_strips > 1 else len(strips[0]))
    ifd += struct.pack(e + "I", 0)
    tail = b"".join(struct.pack(e + "I", o) for o in offs) + b"".join(struct.pack(e + "I", len(s)) for s in strips)
    Path(path).write_bytes(header + ifd + tail + b"".join(strips))


def read_raw(path: Path) -> np.ndarray:
    payload = Path(path).read_bytes()
    assert len(payload) % RAW_DTYPE.itemsize == 0, f"{path}: {len(payload)} bytes"
    return np.frombuffer(payload, dtype=RAW_DTYPE)


def read_manifest(path: Path) -> dict:
    m = json.loads(Path(path).read_text())
    assert m["format"] == "opencorr-gpu-raw-v1" and m["endianness"] == "little" and m["record_bytes"] == 36
    assert isinstance(m["frames"], list)
    return m


def iter_frames(manifest_path: Path):
    m = read_manifest(manifest_path)
    for f in m["frames"]:
        rec = read_raw(Path(manifest_path).parent / (f.get("file") or f["output_name"]))
        assert rec.shape[0] == f["rows"] and rec.nbytes == f["bytes"], f
        yield f, rec


def read_csv(path: Path) -> np.ndarray:
    lines = Path(path).read_text().splitlines()
    assert lines[0] == ",".join(CSV_FIELD_ORDER), lines[0]
    data = np.array([[float(v) for v in ln.split(",")] for ln in lines[1:]]).reshape(-1, 9)
    out = np.zeros(len(data), dtype=RAW_DTYPE)
    for k, name in enumerate(CSV_FIELD_ORDER):
        out[name] = data[:, k]
    return out


def run_cli(binary: Path, args, cwd=None, timeout=600):
    """Runs the command line; returns (exit code, status line dict or None, stderr)."""
    p = subprocess.run([str(binary), *map(str, args)], capture_output=True, text=True, cwd=cwd, timeout=timeout)
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    status = json.loads(lines[-1]) if lines else None
    return p.returncode, status, p.stderr

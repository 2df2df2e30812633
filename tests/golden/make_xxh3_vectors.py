"""Golden XXH3-128 digests for the output ledger's hash.

Runs oracle/_ref/xxh3_ref (the xxHash header the reference vendors, compiled by
oracle/build.py from where it lies in the reference tree) on the xorshift32 byte stream
of oracle/xxh3_check.c for lengths that cover every length class of XXH3-128 and the
1024-byte block boundaries, and writes tests/golden/xxh3_vectors.txt ("<length> <hex>").
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
LENGTHS = [0, 1, 2, 3, 4, 5, 7, 8, 9, 12, 15, 16, 17, 31, 32, 33, 63, 64, 65, 95, 96, 97, 127, 128, 129, 159,
           160, 161, 191, 192, 200, 239, 240, 241, 255, 256, 257, 300, 511, 512, 1000, 1023, 1024, 1025, 1087,
           1088, 1089, 2047, 2048, 2049, 4096, 10000, 65536, 100003]


def main() -> None:
    sys.path.insert(0, str(ROOT))
    from oracle import build
    exe = build.build_xxh3_ref()
    if exe is None:
        raise SystemExit("the reference tree is not present: cannot build oracle/_ref/xxh3_ref")
    out = subprocess.run([str(exe), *map(str, LENGTHS)], check=True, capture_output=True, text=True).stdout
    (HERE / "xxh3_vectors.txt").write_text(out)
    print(f"wrote {len(out.splitlines())} vectors")


if __name__ == "__main__":
    main()

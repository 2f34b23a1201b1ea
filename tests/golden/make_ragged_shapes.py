"""Write ``ragged48_shapes.json``: the 48 (nz, ny, nx) grid shapes of the
ragged-batch workload (sides from {32, 64, 128, 256}, seed 8, seeds
rejected until the batch is within 10 % of 2 GiB of complex64).

    python tests/golden/make_ragged_shapes.py
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "fft3d-fpga_gb300"))

from fftgb.synthetic import ragged_shapes  # noqa: E402


def main() -> None:
    shapes, seed = ragged_shapes()
    total = sum(a * b * c for a, b, c in shapes) * 8
    out = os.path.join(HERE, "ragged48_shapes.json")
    with open(out, "w") as f:
        json.dump({"seed": seed, "bytes": total, "order": "nz, ny, nx",
                   "shapes": [list(s) for s in shapes]}, f)
        f.write("\n")
    print("wrote", out, total, "bytes")


if __name__ == "__main__":
    main()

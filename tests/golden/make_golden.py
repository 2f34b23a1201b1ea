"""Generate the golden 1D vectors from the reference's own FFT engine.

Run where the reference checkout exists (it is compiled in place, nothing is
copied):

    make -C oracle/ref_engine REF=/path/to/fft3d-fpga
    python tests/golden/make_golden.py

Writes ``engine_1d.npz``: for each N in 64..4096 (the sizes the reference's
1D fetch kernel supports, kernels/fft1d/fft1d.cl:48-56) a seeded complex64
input of ``count`` blocks and the engine's forward and inverse outputs, in
the order the reference stores them (bit-reversed within each block).
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.fft_oracle import uniform_c64  # noqa: E402

LIB = os.path.join(ROOT, "oracle", "_ref", "libref_engine.so")


def main() -> None:
    lib = ctypes.CDLL(LIB)
    fn = lib.ref_engine_fft1d
    fn.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_int, ctypes.c_int]
    fn.restype = ctypes.c_int
    arrays = {}
    for log_n in range(6, 13):
        n = 1 << log_n
        count = 3 if n <= 512 else (2 if n <= 1024 else 1)
        x = uniform_c64(n * count, seed=1000 + log_n)
        arrays[f"in_{n}"] = x
        for inv, tag in ((0, "fwd"), (1, "inv")):
            y = np.zeros_like(x)
            rc = fn(log_n, x.ctypes.data, y.ctypes.data, count, inv)
            if rc != 0:
                raise RuntimeError(f"engine failed for N={n}: {rc}")
            arrays[f"{tag}_{n}"] = y
        arrays[f"count_{n}"] = np.array(count)
    out = os.path.join(HERE, "engine_1d.npz")
    np.savez(out, **arrays)
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()

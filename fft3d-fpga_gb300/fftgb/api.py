"""Host-buffer interface mirroring the reference's fftfpga.h entry points.

Each function takes numpy complex64 arrays (host memory, as the reference's
callers pass), calls the identically named C entry point and returns
``(out, timing)`` where ``timing`` is the fpga_t as a dict.  Validation
failures surface as ``timing["valid"] == False`` exactly as in C.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def _c64(x) -> np.ndarray:
    a = np.ascontiguousarray(x, dtype=np.complex64)
    return a


def initialize(platform: str = "NVIDIA CUDA", path: str | None = None,
               use_svm: bool = False) -> int:
    """fpga_initialize (reference api/src/fftfpga.c:72-130)."""
    p = None if path is None else path.encode()
    n = None if platform is None else platform.encode()
    return _lib.lib().fpga_initialize(n, p, use_svm)


def final() -> None:
    """fpga_final (reference api/src/fftfpga.c:135-142)."""
    _lib.lib().fpga_final()


def _run(fn_name: str, x, n_points: int, *args):
    a = _c64(x).reshape(-1)
    if a.size != n_points:
        raise ValueError(f"{fn_name}: expected {n_points} points, got {a.size}")
    out = np.zeros_like(a)
    fn = getattr(_lib.lib(), fn_name)
    t = fn(args[0], a.ctypes.data, out.ctypes.data, *args[1:])
    return out, t.as_dict()


def c2c_1d(x, n: int, inv: bool = False, batch: int = 1, svm: bool = False):
    """fftfpgaf_c2c_1d / _svm: output bit-reversed within each block."""
    name = "fftfpgaf_c2c_1d_svm" if svm else "fftfpgaf_c2c_1d"
    return _run(name, x, n * batch, n, inv, batch)


def c2c_1d_double(x, n: int, inv: bool = False, batch: int = 1):
    """fftfpga_c2c_1d (double2 in/out)."""
    a = np.ascontiguousarray(x, dtype=np.complex128).reshape(-1)
    out = np.zeros_like(a)
    t = _lib.lib().fftfpga_c2c_1d(n, a.ctypes.data, out.ctypes.data, inv, batch)
    return out, t.as_dict()


def c2c_2d_ddr(x, n: int, inv: bool = False):
    return _run("fftfpgaf_c2c_2d_ddr", x, n * n, n, inv)


def c2c_2d_bram(x, n: int, inv: bool = False, how_many: int = 1,
                interleaving: bool = False, svm: bool = False):
    if svm:
        return _run("fftfpgaf_c2c_2d_bram_svm", x, n * n * how_many, n, inv,
                    how_many)
    return _run("fftfpgaf_c2c_2d_bram", x, n * n * how_many, n, inv,
                interleaving, how_many)


def c2c_3d_ddr(x, n: int, inv: bool = False):
    return _run("fftfpgaf_c2c_3d_ddr", x, n ** 3, n, inv)


def c2c_3d_bram(x, n: int, inv: bool = False, interleaving: bool = False):
    return _run("fftfpgaf_c2c_3d_bram", x, n ** 3, n, inv, interleaving)


def c2c_3d_ddr_batch(x, n: int, inv: bool = False, how_many: int = 2,
                     interleaving: bool = False):
    return _run("fftfpgaf_c2c_3d_ddr_batch", x, n ** 3 * how_many, n, inv,
                interleaving, how_many)


def c2c_3d_ddr_svm(x, n: int, inv: bool = False, interleaving: bool = False):
    return _run("fftfpgaf_c2c_3d_ddr_svm", x, n ** 3, n, inv, interleaving)


def c2c_3d_ddr_svm_batch(x, n: int, inv: bool = False, how_many: int = 1):
    return _run("fftfpgaf_c2c_3d_ddr_svm_batch", x, n ** 3 * how_many, n, inv,
                how_many)

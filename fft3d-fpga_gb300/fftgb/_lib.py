"""ctypes binding of libfftfpga.so (the C ABI in include/fftfpga.h and
include/fftfpga_ext.h).

The shared library is built in-tree by ``fft3d-fpga_gb300/build.py``.  There
is no fallback: if the library is missing or fails to load, importing this
module raises.
"""
from __future__ import annotations

import ctypes
import os

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libfftfpga.so")


class Float2(ctypes.Structure):
    """float2 of fftfpga.h (reference api/include/fftfpga/fftfpga.h:16-19)."""
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float)]


class Double2(ctypes.Structure):
    """double2 of fftfpga.h (reference fftfpga.h:24-27)."""
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double)]


class FpgaT(ctypes.Structure):
    """fpga_t of fftfpga.h (reference fftfpga.h:32-39)."""
    _fields_ = [
        ("pcie_read_t", ctypes.c_double),
        ("pcie_write_t", ctypes.c_double),
        ("exec_t", ctypes.c_double),
        ("svm_copyin_t", ctypes.c_double),
        ("svm_copyout_t", ctypes.c_double),
        ("valid", ctypes.c_bool),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Shape3(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_uint), ("ny", ctypes.c_uint), ("nz", ctypes.c_uint)]


# status codes and flags of fftfpga_ext.h
OK = 0
EINVAL = -1
ENODEV = -2
ENOMEM = -3
ECUDA = -4
EUNSUP = -5
ETIMEOUT = -6
ORDER_NATURAL = 0x0
ORDER_BITREV = 0x1
PREC_FP32 = 0x00
PREC_TC_FP16 = 0x10
PREC_TC_BF16 = 0x20
FILTER_POISSON = 1
WAIT_COLS_TMA = 1
WAIT_FUSED_TMA = 2
WAIT_CLUSTER_1D = 3
WAIT_TENSOR_CORE = 4

# every exported entry point with (restype, argtypes)
_u = ctypes.c_uint
_b = ctypes.c_bool
_p = ctypes.c_void_p
_i = ctypes.c_int
_f = ctypes.c_float
_sz = ctypes.c_size_t

SIGNATURES = {
    # fftfpga.h
    "fpga_initialize": (_i, [ctypes.c_char_p, ctypes.c_char_p, _b]),
    "fpga_final": (None, []),
    "fftfpga_complex_malloc": (_p, [_sz]),
    "fftfpgaf_complex_malloc": (_p, [_sz]),
    "fftfpga_c2c_1d": (FpgaT, [_u, _p, _p, _b, _u]),
    "fftfpgaf_c2c_1d": (FpgaT, [_u, _p, _p, _b, _u]),
    "fftfpgaf_c2c_1d_svm": (FpgaT, [_u, _p, _p, _b, _u]),
    "fftfpgaf_c2c_2d_bram": (FpgaT, [_u, _p, _p, _b, _b, _u]),
    "fftfpgaf_c2c_2d_bram_svm": (FpgaT, [_u, _p, _p, _b, _u]),
    "fftfpgaf_c2c_2d_ddr": (FpgaT, [_u, _p, _p, _b]),
    "fftfpgaf_c2c_3d_bram": (FpgaT, [_u, _p, _p, _b, _b]),
    "fftfpgaf_c2c_3d_ddr": (FpgaT, [_u, _p, _p, _b]),
    "fftfpgaf_c2c_3d_ddr_batch": (FpgaT, [_u, _p, _p, _b, _b, _u]),
    "fftfpgaf_c2c_3d_ddr_svm": (FpgaT, [_u, _p, _p, _b, _b]),
    "fftfpgaf_c2c_3d_ddr_svm_batch": (FpgaT, [_u, _p, _p, _b, _u]),
    # fftfpga_ext.h
    "fftgb_plan_1d": (_i, [ctypes.POINTER(_p), _u, _u, _u]),
    "fftgb_plan_2d": (_i, [ctypes.POINTER(_p), _u, _u, _u, _u]),
    "fftgb_plan_3d": (_i, [ctypes.POINTER(_p), _u, _u, _u, _u, _u]),
    "fftgb_plan_destroy": (None, [_p]),
    "fftgb_plan_points": (_sz, [_p]),
    "fftgb_plan_launches": (_i, [_p]),
    "fftgb_plan_inplace_ok": (_i, [_p]),
    "fftgb_exec": (_i, [_p, _p, _p, _i, _f, _p]),
    "fftgb_exec_adjoint": (_i, [_p, _p, _p, _i, _f, _p]),
    "fftgb_exec_filtered": (_i, [_p, _p, _p, _i, _f, _i, _p]),
    "fftgb_exec_adjoint_filtered": (_i, [_p, _p, _p, _i, _f, _i, _p]),
    "fftgb_residual_sq": (_i, [_p, _p, _p, _sz, _p, _p]),
    "fftgb_profile_begin": (_i, [_p, _i]),
    "fftgb_profile_end": (_i, [_p, ctypes.POINTER(ctypes.c_float), _i,
                               ctypes.POINTER(_i)]),
    "fftgb_plan_pass_name": (ctypes.c_char_p, [_p, _i]),
    "fftgb_plan_autotune": (_i, [_p, _i, ctypes.c_char_p, _sz]),
    "fftgb_tune_cache": (_i, [ctypes.c_char_p]),
    "fftgb_plan_variant": (ctypes.c_char_p, [_p]),
    "fftgb_plan_status": (_i, [_p]),
    "fftgb_debug_expire_wait": (_i, [_i, _u]),
    "fftgb_ragged_plan": (_i, [ctypes.POINTER(_p), ctypes.POINTER(Shape3), _u, _u]),
    "fftgb_ragged_destroy": (None, [_p]),
    "fftgb_ragged_points": (_sz, [_p]),
    "fftgb_ragged_exec": (_i, [_p, _p, _p, _i, _p]),
    "fftgb_ragged_launches": (_i, [_p]),
    "fftgb_ragged_status": (_i, [_p]),
    "fftgb_ragged_debug_expire": (_i, [_p, _u]),
    "fftgb_plan_r2c": (_i, [ctypes.POINTER(_p), _i, _u, _u, _u, _u]),
    "fftgb_rplan_destroy": (None, [_p]),
    "fftgb_rplan_real_points": (_sz, [_p]),
    "fftgb_rplan_spectrum_points": (_sz, [_p]),
    "fftgb_exec_r2c": (_i, [_p, _p, _p, _f, _p]),
    "fftgb_exec_c2r": (_i, [_p, _p, _p, _f, _p]),
    "fftgb_c2c_1d_noalloc": (_i, [_u, _u, _p, _p, _i, _p]),
    "fftgb_noalloc_last_error": (ctypes.c_char_p, []),
    "fftgb_tc_selftest": (_i, [_i, ctypes.POINTER(ctypes.c_float)]),
    "fftgb_last_error": (ctypes.c_char_p, []),
    "fftgb_version": (ctypes.c_char_p, []),
}


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    if not os.path.exists(path):
        raise RuntimeError(
            f"libfftfpga.so not found at {path}; build it with "
            "`python fft3d-fpga_gb300/build.py` (there is no CPU fallback)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_LIB = None


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = load()
    return _LIB


def last_error() -> str:
    return lib().fftgb_last_error().decode()


class FFTGBError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what} failed with status {code}: {last_error()}")
        self.code = code


def check(code: int, what: str) -> None:
    if code != OK:
        raise FFTGBError(code, what)

"""Device-tensor plans over the extension ABI (include/fftfpga_ext.h).

torch is used only as plumbing: it owns device memory and streams; every
transform runs in libfftfpga.so's own kernels.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib

_PREC = {"fp32": _lib.PREC_FP32, "tc_fp16": _lib.PREC_TC_FP16,
         "tc_bf16": _lib.PREC_TC_BF16}


def _stream_ptr(stream) -> int:
    s = torch.cuda.current_stream() if stream is None else stream
    return int(s.cuda_stream)


class Plan:
    """Batched C2C plan for grids of shape ``dims`` (slowest first: (n,),
    (ny, nx) or (nz, ny, nx)) on complex64 CUDA tensors."""

    def __init__(self, dims, batch: int = 1, order: str = "natural",
                 precision: str = "fp32"):
        dims = tuple(int(d) for d in dims)
        if not 1 <= len(dims) <= 3:
            raise ValueError("rank must be 1, 2 or 3")
        self.dims = dims
        self.batch = int(batch)
        flags = _PREC[precision]
        if order == "bitrev":
            flags |= _lib.ORDER_BITREV
        elif order != "natural":
            raise ValueError(order)
        self.flags = flags
        h = ctypes.c_void_p()
        L = _lib.lib()
        if len(dims) == 1:
            rc = L.fftgb_plan_1d(ctypes.byref(h), dims[0], self.batch, flags)
        elif len(dims) == 2:
            rc = L.fftgb_plan_2d(ctypes.byref(h), dims[1], dims[0], self.batch, flags)
        else:
            rc = L.fftgb_plan_3d(ctypes.byref(h), dims[2], dims[1], dims[0],
                                 self.batch, flags)
        _lib.check(rc, "fftgb_plan")
        self._h = h
        self.points = int(L.fftgb_plan_points(h))
        self.launches = int(L.fftgb_plan_launches(h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().fftgb_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    def _check(self, x: torch.Tensor) -> None:
        if x.dtype != torch.complex64 or not x.is_cuda:
            raise TypeError("expected a complex64 CUDA tensor")
        if not x.is_contiguous():
            raise ValueError("expected a contiguous tensor")
        if x.numel() != self.points:
            raise ValueError(f"expected {self.points} points, got {x.numel()}")

    def execute(self, x: torch.Tensor, inverse: bool = False, scale: float = 1.0,
                out: torch.Tensor | None = None, stream=None,
                adjoint: bool = False, filter: str | None = None) -> torch.Tensor:
        """Transform (or its adjoint) of ``x``; ``filter="poisson"``
        multiplies the outputs by G = 1/|k|^2 (G(0) = 0) in the same call
        (3D plans)."""
        self._check(x)
        if out is None:
            out = torch.empty_like(x)
        self._check(out)
        L = _lib.lib()
        if filter is None:
            fn = L.fftgb_exec_adjoint if adjoint else L.fftgb_exec
            rc = fn(self._h, x.data_ptr(), out.data_ptr(), 1 if inverse else 0,
                    float(scale), _stream_ptr(stream))
        else:
            if filter != "poisson":
                raise ValueError(filter)
            fn = L.fftgb_exec_adjoint_filtered if adjoint else L.fftgb_exec_filtered
            rc = fn(self._h, x.data_ptr(), out.data_ptr(), 1 if inverse else 0,
                    float(scale), _lib.FILTER_POISSON, _stream_ptr(stream))
        _lib.check(rc, "fftgb_exec" + ("_adjoint" if adjoint else "")
                   + ("_filtered" if filter else ""))
        return out

    def __call__(self, x, inverse=False, scale=1.0, out=None, stream=None):
        return self.execute(x, inverse, scale, out, stream)

    def autotune(self, reps: int = 5) -> str:
        """Time every decomposition of this shape, keep the fastest; returns
        the timing report."""
        buf = ctypes.create_string_buffer(2048)
        _lib.check(_lib.lib().fftgb_plan_autotune(self._h, int(reps), buf,
                                                  len(buf)),
                   "fftgb_plan_autotune")
        self.launches = int(_lib.lib().fftgb_plan_launches(self._h))
        return buf.value.decode()

    def status(self) -> int:
        """0, or -6 (timeout) if a bounded device-side wait of the plan's
        kernels gave up since the last call (synchronises, clears it)."""
        return int(_lib.lib().fftgb_plan_status(self._h))

    @property
    def variant(self) -> str:
        return _lib.lib().fftgb_plan_variant(self._h).decode()

    def pass_names(self) -> list[str]:
        L = _lib.lib()
        return [L.fftgb_plan_pass_name(self._h, i).decode()
                for i in range(self.launches)]

    def profile_begin(self, max_execs: int) -> None:
        _lib.check(_lib.lib().fftgb_profile_begin(self._h, int(max_execs)),
                   "fftgb_profile_begin")

    def profile_end(self) -> tuple[list[float], int]:
        """Summed CUDA-event milliseconds per pass, and executions recorded."""
        ms = (ctypes.c_float * self.launches)()
        n = ctypes.c_int()
        _lib.check(_lib.lib().fftgb_profile_end(self._h, ms, self.launches,
                                                ctypes.byref(n)),
                   "fftgb_profile_end")
        return list(ms), n.value


class RaggedPlan:
    """Ragged batch of 3D grids given as (nz, ny, nx) tuples, packed back to
    back in one complex64 CUDA tensor."""

    def __init__(self, shapes, precision: str = "fp32"):
        arr = (_lib.Shape3 * len(shapes))()
        for i, (nz, ny, nx) in enumerate(shapes):
            arr[i].nx, arr[i].ny, arr[i].nz = int(nx), int(ny), int(nz)
        h = ctypes.c_void_p()
        rc = _lib.lib().fftgb_ragged_plan(ctypes.byref(h), arr, len(shapes),
                                          _PREC[precision])
        _lib.check(rc, "fftgb_ragged_plan")
        self._h = h
        self.shapes = [tuple(s) for s in shapes]
        self.points = int(_lib.lib().fftgb_ragged_points(h))
        self.launches = int(_lib.lib().fftgb_ragged_launches(h))

    def status(self) -> int:
        """0, or -6 (timeout) if a dependency wait gave up (synchronises)."""
        return int(_lib.lib().fftgb_ragged_status(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().fftgb_ragged_destroy(h)
            except Exception:
                pass
            self._h = None

    def __call__(self, x: torch.Tensor, inverse: bool = False,
                 out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        if x.dtype != torch.complex64 or not x.is_cuda or x.numel() != self.points:
            raise ValueError("bad ragged input")
        if out is None:
            out = torch.empty_like(x)
        rc = _lib.lib().fftgb_ragged_exec(self._h, x.data_ptr(), out.data_ptr(),
                                          1 if inverse else 0, _stream_ptr(stream))
        _lib.check(rc, "fftgb_ragged_exec")
        return out


class RealPlan:
    """Real-data plan over real grids of shape ``dims`` (slowest first) and
    their half spectra (last axis dims[-1] // 2 + 1): ``r2c`` float32 ->
    complex64, ``c2r`` complex64 -> float32 (unnormalised)."""

    def __init__(self, dims, batch: int = 1):
        dims = tuple(int(d) for d in dims)
        if not 1 <= len(dims) <= 3:
            raise ValueError("rank must be 1, 2 or 3")
        full = (1,) * (3 - len(dims)) + dims  # (nz, ny, nx)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().fftgb_plan_r2c(ctypes.byref(h), len(dims), full[2],
                                             full[1], full[0], int(batch)),
                   "fftgb_plan_r2c")
        self._h = h
        self.dims = dims
        self.batch = int(batch)
        self.real_points = int(_lib.lib().fftgb_rplan_real_points(h))
        self.spectrum_points = int(_lib.lib().fftgb_rplan_spectrum_points(h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.lib().fftgb_rplan_destroy(h)
            except Exception:
                pass
            self._h = None

    @staticmethod
    def _dev(x, dtype, n):
        if x.dtype != dtype or not x.is_cuda or not x.is_contiguous() or x.numel() != n:
            raise ValueError(f"expected a contiguous {dtype} CUDA tensor of {n} elements")

    def r2c(self, x: torch.Tensor, out: torch.Tensor | None = None, scale: float = 1.0,
            stream=None) -> torch.Tensor:
        self._dev(x, torch.float32, self.real_points)
        if out is None:
            out = torch.empty(self.spectrum_points, dtype=torch.complex64, device=x.device)
        self._dev(out, torch.complex64, self.spectrum_points)
        _lib.check(_lib.lib().fftgb_exec_r2c(self._h, x.data_ptr(), out.data_ptr(),
                                             float(scale), _stream_ptr(stream)),
                   "fftgb_exec_r2c")
        return out

    def c2r(self, x: torch.Tensor, out: torch.Tensor | None = None, scale: float = 1.0,
            stream=None) -> torch.Tensor:
        self._dev(x, torch.complex64, self.spectrum_points)
        if out is None:
            out = torch.empty(self.real_points, dtype=torch.float32, device=x.device)
        self._dev(out, torch.float32, self.real_points)
        _lib.check(_lib.lib().fftgb_exec_c2r(self._h, x.data_ptr(), out.data_ptr(),
                                             float(scale), _stream_ptr(stream)),
                   "fftgb_exec_c2r")
        return out

"""FP64 oracle for the FFTFPGA single-precision C2C path.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by ``__graft_entry__.smoke()``
to verify its results and by ``bench.py``'s CPU-baseline leg.  The product library
never imports, links or executes anything in this folder.

It restates what the reference computes, in complex128 with numpy's
pocketfft, so that every GPU result can be compared against it:

* sign: forward uses exp(-2*pi*i*n*k/N)             (kernels/common/fft_8.cl:240,
  twiddle tables kernels/common/twid_radix4_8.cl:60-89 hold -sin)
* inverse is the *unnormalised* backward transform  (fft_8.cl:276-278, 341-343,
  matching FFTW_BACKWARD in examples/helper.cpp:133-135)
* 1D output order is bit-reversed within each N-point block
  (fft_8.cl:28-30, kernels/fft1d/fft1d.cl:236-250, undone by the
  reference's own check in examples/helper.cpp:143-162)
* 2D/3D outputs are in natural order, row-major with x fastest and the
  batch index slowest (kernels/fft3d/fft3d_ddr.cl:479-485,
  api/src/fft3d.c:396-913 places grid i at inp[i*N^3])
* accuracy metric: the reference's SNR in dB (examples/helper.cpp:164-198,
  pass above 120 dB) and the relative L2 error, both accumulated in FP64.

Parity pin: ``tests/golden/`` holds vectors produced by the reference's own
FFT engine (kernels/common/fft_8.cl compiled in place, see
oracle/ref_engine/); ``tests/test_oracle.py`` checks this module against them.
"""
from __future__ import annotations

import os

import numpy as np

__all__ = [
    "bitrev_perm",
    "c2c_1d",
    "c2c_nd",
    "dft_direct",
    "rel_l2",
    "snr_db",
    "uniform_c64",
]


def bitrev_perm(log_n: int) -> np.ndarray:
    """Index permutation j -> bit_reversed(j, log_n).

    Same mapping as ``bit_reversed`` in examples/helper.cpp:10-18 and
    kernels/fft1d/fft1d.cl:67-76.
    """
    n = 1 << log_n
    j = np.arange(n, dtype=np.int64)
    r = np.zeros(n, dtype=np.int64)
    for b in range(log_n):
        r |= ((j >> b) & 1) << (log_n - 1 - b)
    return r


def _as_c128(x) -> np.ndarray:
    return np.asarray(x).astype(np.complex128, copy=False)


def c2c_nd(x, shape, inverse: bool = False, batch: int = 1) -> np.ndarray:
    """Natural-order D-dimensional C2C FFT of ``batch`` grids, in FP64.

    ``shape`` is given slowest-first, e.g. (nz, ny, nx) for a 3D grid, which
    is how the reference lays grids out (x fastest).  The inverse is not
    normalised.  Follows api/src/fft2d.c:27-159 and api/src/fft3d.c:206-384.
    """
    shape = tuple(int(s) for s in shape)
    a = _as_c128(x).reshape((batch,) + shape)
    axes = tuple(range(1, len(shape) + 1))
    try:  # same pocketfft algorithm in FP64, threaded for large grids
        import scipy.fft as sf
        workers = len(os.sched_getaffinity(0))
        if inverse:
            y = sf.ifftn(a, axes=axes, norm="forward", workers=workers)
        else:
            y = sf.fftn(a, axes=axes, workers=workers)
    except ImportError:  # pragma: no cover
        if inverse:
            n = int(np.prod(shape))
            y = np.fft.ifftn(a, axes=axes) * n
        else:
            y = np.fft.fftn(a, axes=axes)
    return y.reshape(-1)


def r2c_nd(x, shape, batch: int = 1) -> np.ndarray:
    """Half spectrum (last axis n // 2 + 1) of ``batch`` real grids of
    ``shape`` (slowest first), sign -, in FP64.  The reference has no
    real-data transform; this is the half-spectrum convention of FFTW, the
    library its verifier uses (examples/helper.cpp:119-141)."""
    shape = tuple(int(s) for s in shape)
    a = np.asarray(x, dtype=np.float64).reshape((batch,) + shape)
    axes = tuple(range(1, len(shape) + 1))
    return np.fft.rfftn(a, axes=axes).reshape(-1)


def c2r_nd(spec, shape, batch: int = 1) -> np.ndarray:
    """Unnormalised inverse of r2c_nd (sign +): real grids of ``shape``
    scaled by their point count, in FP64.  Only the Hermitian part of the
    input is used (imaginary parts of the self-conjugate bins are ignored)."""
    shape = tuple(int(s) for s in shape)
    half = shape[:-1] + (shape[-1] // 2 + 1,)
    a = _as_c128(spec).reshape((batch,) + half)
    axes = tuple(range(1, len(shape) + 1))
    return (np.fft.irfftn(a, s=shape, axes=axes) * int(np.prod(shape))).reshape(-1)


def c2c_1d(x, n: int, inverse: bool = False, batch: int = 1,
           bit_reversed: bool = True) -> np.ndarray:
    """1D C2C FFT of ``batch`` contiguous N-point blocks, in FP64.

    With ``bit_reversed`` (the fftfpgaf_c2c_1d ABI, api/src/fft1d.c:148-247)
    output position j of each block holds X[bit_reversed(j)].
    """
    y = c2c_nd(x, (n,), inverse, batch).reshape(batch, n)
    if bit_reversed:
        y = y[:, bitrev_perm(int(n).bit_length() - 1)]
    return y.reshape(-1)


def dft_direct(x, inverse: bool = False) -> np.ndarray:
    """O(N^2) FP64 DFT along the last axis, for cross-checking pocketfft."""
    a = _as_c128(x)
    n = a.shape[-1]
    k = np.arange(n)
    sgn = 1.0 if inverse else -1.0
    w = np.exp(sgn * 2j * np.pi * np.outer(k, k) / n)
    return a @ w.T


def rel_l2(y, y_ref) -> float:
    """||y - y_ref||_2 / ||y_ref||_2, accumulated in FP64."""
    a = _as_c128(y).reshape(-1)
    b = _as_c128(y_ref).reshape(-1)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a))


def snr_db(y, y_ref) -> float:
    """Reference-style SNR: 10 log10(sum|ref|^2 / sum|ref - y|^2).

    examples/helper.cpp:164-198 (accumulated there in FP32; FP64 here).
    """
    a = _as_c128(y).reshape(-1)
    b = _as_c128(y_ref).reshape(-1)
    noise = float(np.sum(np.abs(b - a) ** 2))
    sig = float(np.sum(np.abs(b) ** 2))
    if noise == 0.0:
        return float("inf")
    return 10.0 * np.log10(sig / noise)


def uniform_c64(count: int, seed: int) -> np.ndarray:
    """Seeded complex64 with i.i.d. U[-1, 1) real and imaginary parts."""
    rng = np.random.default_rng(seed)
    re = rng.uniform(-1.0, 1.0, count).astype(np.float32)
    im = rng.uniform(-1.0, 1.0, count).astype(np.float32)
    out = np.empty(count, dtype=np.complex64)
    out.real = re
    out.imag = im
    return out

"""CPU baseline for the FFT path (test/benchmark infrastructure only).

The reference's CPU path is FFTW single precision (examples/helper.cpp:
119-141, fftwf_plan_many_dft).  FFTW is not installed on either machine, so
the baseline is the oracle's CPU FFT port: pocketfft (scipy.fft) on
complex64, threaded over every host core this process may use, out of place,
plan/warm-up excluded.  Only bench.py's CPU-baseline leg and its reference
arm call this module; the product library never does.
"""
from __future__ import annotations

import os
import time

import numpy as np


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


def fft_c64(x: np.ndarray, axes, inverse: bool, workers: int) -> np.ndarray:
    import scipy.fft as sf
    if inverse:
        return sf.ifftn(x, axes=axes, norm="forward", workers=workers)
    return sf.fftn(x, axes=axes, workers=workers)


def time_transform(shape, batch: int, reps: int, workers: int | None = None,
                   seed: int = 0, directions=(False, True)) -> dict:
    """Median seconds per (forward + inverse) step over ``reps`` runs on a
    ``batch`` of complex64 grids of ``shape`` (slowest first)."""
    workers = workers or host_cores()
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape)) * batch
    x = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(np.complex64)
    x = x.reshape((batch,) + tuple(shape))
    axes = tuple(range(1, len(shape) + 1))
    for inv in directions:  # warm-up (plan caches, page faults)
        fft_c64(x, axes, inv, workers)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        for inv in directions:
            y = fft_c64(x, axes, inv, workers)
        times.append(time.perf_counter() - t0)
        assert y.dtype == np.complex64
    times.sort()
    return {"seconds": times[len(times) // 2], "workers": workers,
            "points": n, "reps": reps}

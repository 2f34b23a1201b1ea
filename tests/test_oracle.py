"""The FP64 oracle, pinned against the reference's own FFT engine.

tests/golden/engine_1d.npz holds outputs of the reference's radix-2^2 engine
(kernels/common/fft_8.cl compiled in place by oracle/ref_engine, driven as
the fft1d task drives it).  The reference's own pass rule is an SNR above
120 dB against a single-precision FFT (examples/helper.cpp:164-198); here the
oracle must reproduce the engine's outputs - including the bit-reversed
order, the forward sign and the unnormalised inverse - to that level.
"""
import os

import numpy as np
import pytest

from oracle import fft_oracle as orc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "engine_1d.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("log_n", range(6, 13))
@pytest.mark.parametrize("inv", [False, True])
def test_oracle_matches_reference_engine(golden, log_n, inv):
    n = 1 << log_n
    x = golden[f"in_{n}"]
    count = int(golden[f"count_{n}"])
    y_eng = golden[f"{'inv' if inv else 'fwd'}_{n}"]
    y_orc = orc.c2c_1d(x, n, inverse=inv, batch=count, bit_reversed=True)
    assert orc.snr_db(y_eng, y_orc) > 120.0
    assert orc.rel_l2(y_eng, y_orc) < 1e-6


def test_golden_order_is_not_natural(golden):
    # the pin must be able to fail: natural order misses by O(1)
    n = 256
    x = golden[f"in_{n}"]
    count = int(golden[f"count_{n}"])
    y_nat = orc.c2c_1d(x, n, batch=count, bit_reversed=False)
    assert orc.rel_l2(golden[f"fwd_{n}"], y_nat) > 0.5


def test_golden_sign_and_scale(golden):
    n = 512
    x = golden[f"in_{n}"]
    count = int(golden[f"count_{n}"])
    # wrong sign: forward engine output vs oracle inverse
    y_wrong = orc.c2c_1d(x, n, inverse=True, batch=count)
    assert orc.rel_l2(golden[f"fwd_{n}"], y_wrong) > 0.5
    # normalised inverse would be off by a factor N
    y_norm = orc.c2c_1d(x, n, inverse=True, batch=count) / n
    assert orc.rel_l2(golden[f"inv_{n}"], y_norm) > 0.5


@pytest.mark.parametrize("n", [2, 8, 64, 256])
@pytest.mark.parametrize("inv", [False, True])
def test_pocketfft_vs_direct_dft(n, inv):
    x = orc.uniform_c64(n * 3, seed=n).reshape(3, n)
    a = orc.c2c_nd(x, (n,), inverse=inv, batch=3).reshape(3, n)
    b = orc.dft_direct(x, inverse=inv)
    assert orc.rel_l2(a, b) < 1e-12


@pytest.mark.parametrize("n", [3, 5, 6, 7, 12, 15, 96, 100, 240])
@pytest.mark.parametrize("inv", [False, True])
def test_pocketfft_vs_direct_dft_not_power_of_two(n, inv):
    """The oracle of the non-power-of-two extension (mixed-radix and
    Bluestein plans) against the direct FP64 DFT."""
    x = orc.uniform_c64(n * 3, seed=n).reshape(3, n)
    a = orc.c2c_nd(x, (n,), inverse=inv, batch=3).reshape(3, n)
    b = orc.dft_direct(x, inverse=inv)
    assert orc.rel_l2(a, b) < 1e-12


def test_nd_not_power_of_two_matches_separable_direct():
    x = orc.uniform_c64(6 * 5 * 12, seed=8).reshape(6, 5, 12)
    y = orc.c2c_nd(x, (6, 5, 12)).reshape(6, 5, 12)
    z = orc.dft_direct(x)
    z = np.swapaxes(orc.dft_direct(np.swapaxes(z, 1, 2)), 1, 2)
    z = np.swapaxes(orc.dft_direct(np.swapaxes(z, 0, 2)), 0, 2)
    assert orc.rel_l2(y, z) < 1e-12


@pytest.mark.parametrize("shape", [(12,), (6, 10), (3, 5, 6), (4, 8)])
def test_r2c_c2r_vs_direct_dft(shape):
    """The real-data oracle (half spectrum, unnormalised inverse) against the
    direct DFT of the real grid, even and odd outer sides included."""
    n = int(np.prod(shape))
    x = np.random.default_rng(n).uniform(-1, 1, n * 2)
    spec = orc.r2c_nd(x, shape, 2).reshape((2,) + shape[:-1] + (shape[-1] // 2 + 1,))
    full = x.reshape((2,) + shape).astype(np.complex128)
    for ax in range(1, len(shape) + 1):
        full = np.swapaxes(orc.dft_direct(np.swapaxes(full, ax, -1)), ax, -1)
    assert orc.rel_l2(spec, full[..., : shape[-1] // 2 + 1]) < 1e-12
    back = orc.c2r_nd(spec.reshape(-1), shape, 2)
    assert orc.rel_l2(back, n * x) < 1e-12


def test_nd_matches_separable_direct():
    x = orc.uniform_c64(8 * 4 * 16, seed=7).reshape(8, 4, 16)
    y = orc.c2c_nd(x, (8, 4, 16)).reshape(8, 4, 16)
    z = orc.dft_direct(x)                                     # x axis
    z = np.swapaxes(orc.dft_direct(np.swapaxes(z, 1, 2)), 1, 2)  # y axis
    z = np.swapaxes(orc.dft_direct(np.swapaxes(z, 0, 2)), 0, 2)  # z axis
    assert orc.rel_l2(y, z) < 1e-12


def test_analytic_cases():
    n = 64
    d = np.zeros(n, np.complex64)
    d[0] = 1
    assert np.allclose(orc.c2c_nd(d, (n,)), np.ones(n))
    k0 = 5
    tone = np.exp(-2j * np.pi * k0 * np.arange(n) / n * -1)  # e^{+2 pi i k0 n/N}
    y = orc.c2c_nd(tone, (n,))
    e = np.zeros(n)
    e[k0] = n
    assert np.allclose(y, e, atol=1e-9)


def test_bitrev_perm_is_involution():
    for lg in range(0, 13):
        p = orc.bitrev_perm(lg)
        assert np.array_equal(p[p], np.arange(1 << lg))


def test_metrics():
    a = np.ones(10, np.complex128)
    assert orc.rel_l2(a, a) == 0.0
    assert orc.snr_db(a, a) == float("inf")
    b = a * (1 + 1e-6)
    assert abs(orc.snr_db(b, a) - 120.0) < 0.01

"""Real-data transforms (R2C / C2R; no reference counterpart) against the
FP64 oracle: rel-L2 <= 2e-6 for the forward half spectrum, C2R of an exact
half spectrum against N x, and round trips; batches, 1D/2D/3D, the smallest
and largest row lengths, lengths 2^a 3^b 5^c, scaling, and rejected
arguments."""
import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _real(n, seed):
    return np.random.default_rng(seed).uniform(-1, 1, n).astype(np.float32)


@pytest.mark.parametrize("dims,batch", [
    ((4,), 3), ((16,), 5), ((1024,), 7), ((8192,), 2),
    ((64, 128), 3), ((1024, 1024), 1), ((8, 4), 2), ((4096, 32), 1),
    ((32, 32, 32), 2), ((64, 128, 256), 1), ((16, 8, 4), 3), ((128, 128, 128), 2),
])
def test_r2c_c2r(cuda, dims, batch):
    _check_r2c_c2r(cuda, dims, batch)


@pytest.mark.parametrize("dims,batch", [
    ((6,), 5), ((10,), 3), ((12,), 4), ((96,), 7), ((100,), 3), ((1000,), 5), ((6000,), 2),
    ((8000,), 1), ((96, 100), 2), ((100, 64), 3), ((64, 96), 2), ((30, 50), 4), ((3, 8), 2),
    ((96, 96, 96), 2), ((16, 12, 10), 3), ((45, 27, 64), 1), ((64, 64, 96), 1),
    ((96, 64, 64), 1), ((5, 6, 20), 3), ((120, 120, 120), 1), ((20, 1000), 2),
    ((6, 8, 960), 2),
])
def test_r2c_c2r_not_power_of_two(cuda, dims, batch):
    """Axis lengths 2^a 3^b 5^c (nx/2 of that form): the mixed-radix passes,
    the x pass over the real rows packed as nx/2 complex points plus the
    untangle (C2R: tangle) pass."""
    _check_r2c_c2r(cuda, dims, batch)


@pytest.mark.parametrize("dims,batch", [((96,), 3), ((64, 100), 2), ((30, 24, 36), 2)])
def test_r2c_c2r_generic_kernel(cuda, monkeypatch, dims, batch):
    """FFTGB_MIX_GENERIC=1: the mixed-radix passes through the kernel that
    holds every radix instead of the two- and three-stage instantiations."""
    monkeypatch.setenv("FFTGB_MIX_GENERIC", "1")
    _check_r2c_c2r(cuda, dims, batch)


def _check_r2c_c2r(cuda, dims, batch):
    import torch
    from fftgb.plan import RealPlan
    p = RealPlan(dims, batch)
    n = int(np.prod(dims))
    assert p.real_points == n * batch
    assert p.spectrum_points == n // dims[-1] * (dims[-1] // 2 + 1) * batch
    x = _real(n * batch, seed=n + batch)
    xd = torch.from_numpy(x).to(cuda)
    spec = p.r2c(xd).cpu().numpy()
    ref = orc.r2c_nd(x, dims, batch)
    assert orc.rel_l2(spec, ref) <= TOL
    # C2R of the exact (FP64-computed) half spectrum
    sd = torch.from_numpy(ref.astype(np.complex64)).to(cuda)
    y = p.c2r(sd).cpu().numpy()
    assert orc.rel_l2(y, orc.c2r_nd(ref, dims, batch)) <= TOL
    assert orc.rel_l2(y, n * x.astype(np.float64)) <= TOL
    # the input of C2R is not modified
    assert np.array_equal(sd.cpu().numpy(), ref.astype(np.complex64))
    # round trip with the 1/N scale on the way back
    z = p.c2r(p.r2c(xd), scale=1.0 / n).cpu().numpy()
    assert orc.rel_l2(z, x) <= 2 * TOL


@pytest.mark.parametrize("dims", [(256,), (32, 64), (16, 16, 16)])
def test_r2c_scale(cuda, dims):
    import torch
    from fftgb.plan import RealPlan
    p = RealPlan(dims, 2)
    x = _real(int(np.prod(dims)) * 2, seed=5)
    y = p.r2c(torch.from_numpy(x).to(cuda), scale=0.25).cpu().numpy()
    assert orc.rel_l2(y, 0.25 * orc.r2c_nd(x, dims, 2)) <= TOL


def test_real_plan_rejects(cuda):
    from fftgb import FFTGBError
    from fftgb.plan import RealPlan
    for dims in [(2,), (14,), (15,), (22,), (16384,), (16, 16384), (8192, 16, 16), (7, 16),
                 (16, 7, 16), (12000,)]:
        with pytest.raises(FFTGBError):
            RealPlan(dims, 1)
    with pytest.raises(FFTGBError):
        RealPlan((64,), 0)

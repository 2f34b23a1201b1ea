"""Tensor-core split-precision form.

* building block: the tcgen05 MMA with shared-memory operands in the
  core-matrix layout and FP32 accumulators read back from TMEM reproduces an
  FP64 product of half-precision-exact inputs;
* the FFT plans whose radix-16 stages run on the tensor cores (split FP16,
  3 products; split BF16, 6 products) meet the plain FP32 form's bound,
  rel-L2 <= 2e-6 against the FP64 oracle, on uniform inputs and on a
  plane-wave-density-like input with ~1e6 dynamic range.
"""
import ctypes

import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6


@pytest.mark.parametrize("bf16", [0, 1])
def test_tcgen05_selftest(lib, cuda, bf16):
    err = ctypes.c_float(-1.0)
    rc = lib.fftgb_tc_selftest(bf16, ctypes.byref(err))
    assert rc == 0, lib.fftgb_last_error()
    assert 0.0 <= err.value < 1e-6, err.value


def _run(cuda, dims, batch, prec, x, inverse=False):
    import torch
    from fftgb.plan import Plan
    p = Plan(dims, batch, precision=prec)
    names = p.pass_names()
    y = p(torch.from_numpy(x).to(cuda), inverse=inverse).cpu().numpy()
    assert p.status() == 0  # no MMA completion wait gave up
    return y, names


@pytest.mark.parametrize("prec", ["tc_fp16", "tc_bf16"])
@pytest.mark.parametrize("dims,batch", [((512,), 64), ((256, 256), 3),
                                        ((256, 256, 256), 1)])
def test_tc_fft_uniform(cuda, prec, dims, batch):
    x = orc.uniform_c64(int(np.prod(dims)) * batch, seed=31)
    for inv in (False, True):
        y, names = _run(cuda, dims, batch, prec, x, inv)
        assert any("_tc<" in n for n in names), names
        err = orc.rel_l2(y, orc.c2c_nd(x, dims, inv, batch))
        assert err <= TOL, (prec, dims, inv, err)


@pytest.mark.parametrize("prec", ["tc_fp16", "tc_bf16"])
def test_tc_fft_plane_wave_density(cuda, prec):
    from fftgb import synthetic
    dims = (256, 256, 256)
    x = synthetic.plane_wave_density(dims, seed=7)
    y, names = _run(cuda, dims, 1, prec, x)
    ref = orc.c2c_nd(x, dims)
    # the input's Fourier amplitudes span ~1e6 (scaled by (1 + |k|^2)^-2)
    mag = np.abs(ref)
    assert mag.max() / np.percentile(mag, 50) > 1e5
    assert orc.rel_l2(y, ref) <= TOL


def test_tc_512_cubed_forward(cuda):
    """512^3 (the precision-form workload) against the FP64 oracle."""
    import torch
    from fftgb.plan import Plan
    n = 512
    x = orc.uniform_c64(n ** 3, seed=6)
    for prec in ("tc_fp16", "tc_bf16"):
        p = Plan((n, n, n), 1, precision=prec)
        y = p(torch.from_numpy(x).to(cuda)).cpu().numpy()
        assert orc.rel_l2(y, orc.c2c_nd(x, (n, n, n))) <= TOL, prec
        del p
        torch.cuda.empty_cache()


def test_tc_512_cubed_round_trip(cuda):
    import torch
    from fftgb.plan import Plan
    n = 512
    p = Plan((n, n, n), 1, precision="tc_fp16")
    g = torch.Generator(device=cuda).manual_seed(6)
    x = torch.view_as_complex((torch.rand(p.points, 2, device=cuda, generator=g) * 2 - 1).contiguous())
    y = p(x)
    xs = x.view(n, n, n).sum(0).cpu().numpy().astype(np.complex128)
    assert orc.rel_l2(y.view(n, n, n)[0].cpu().numpy(), np.fft.fft2(xs)) <= 4 * TOL
    z = p(y, inverse=True, scale=1.0 / n ** 3)
    err = ((z - x).abs() ** 2).double().sum().sqrt() / (x.abs() ** 2).double().sum().sqrt()
    assert err.item() <= 2 * TOL  # two transforms

"""Axis lengths that are not powers of two (Bluestein's algorithm; no
reference counterpart, the reference takes powers of two only): 1D, 2D, 3D
and mixed grids against the FP64 oracle at rel-L2 <= 2e-6, both directions,
scaling, in place, and the rejected cases."""
import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _run(cuda, dims, batch, inplace=False, scale=1.0):
    import torch
    from fftgb.plan import Plan
    p = Plan(dims, batch)
    assert p.variant == "bluestein"
    x = orc.uniform_c64(p.points, seed=sum(dims) + batch)
    for inv in (False, True):
        xd = torch.from_numpy(x).to(cuda)
        y = p(xd, inverse=inv, scale=scale, out=xd if inplace else None).cpu().numpy()
        ref = scale * orc.c2c_nd(x, dims, inv, batch)
        assert orc.rel_l2(y, ref) <= TOL, (dims, inv, p.pass_names())
    return p


@pytest.mark.parametrize("n", [3, 5, 6, 7, 12, 100, 125, 243, 1000, 1536, 2047])
def test_1d(cuda, n):
    _run(cuda, (n,), 3)


@pytest.mark.parametrize("dims,batch", [
    ((60, 100), 2), ((1000, 48), 1), ((100, 64), 3), ((64, 100), 2), ((7, 9), 5),
])
def test_2d(cuda, dims, batch):
    _run(cuda, dims, batch)


@pytest.mark.parametrize("dims,batch", [
    ((27, 45, 64), 1), ((16, 12, 10), 3), ((125, 125, 125), 1), ((96, 96, 96), 1),
    ((64, 64, 3), 2),
])
def test_3d(cuda, dims, batch):
    p = _run(cuda, dims, batch)
    names = p.pass_names()
    assert any(n.startswith("k_blue") for n in names), names


def test_scale_and_in_place(cuda):
    _run(cuda, (30, 50), 2, inplace=True, scale=0.125)


def test_rejected(cuda):
    from fftgb import FFTGBError
    from fftgb.plan import Plan
    for args, kw in [(((2049,), 1), {}), (((100,), 1), {"order": "bitrev"}),
                     (((100,), 1), {"precision": "tc_fp16"}), (((8192, 3), 1), {})]:
        with pytest.raises(FFTGBError):
            Plan(*args, **kw)

"""Full-size configurations checked over every point against the FP64
oracle (rel-L2 <= 2e-6, accumulated over the whole batch):

* 256^3 x 8 (1 GiB, the headline), forward and unnormalised inverse over
  all eight grids, device-pointer plan and the
  fftfpgaf_c2c_3d_ddr_batch(how_many = 8) entry point on host buffers, plus
  Parseval's identity per grid (sum |X|^2 = N sum |x|^2);
* 512^3 x 1 (1 GiB), forward and unnormalised inverse, device-pointer plan
  and the fftfpgaf_c2c_3d_ddr entry point on host buffers;
* 2D 1024^2 x 64 (512 MiB), forward and inverse, plan and
  fftfpgaf_c2c_2d_bram(how_many = 64);
* 1D 65536 x 1024 (512 MiB), natural-order plan and the bit-reversed
  fftfpgaf_c2c_1d entry point.

The oracle's FP64 FFT of these sizes takes a few seconds on the host cores.
"""
import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _plan_both_directions(cuda, dims, batch, seed):
    import torch
    from fftgb.plan import Plan
    p = Plan(dims, batch)
    x = orc.uniform_c64(p.points, seed=seed)
    xd = torch.from_numpy(x).to(cuda)
    for inv in (False, True):
        y = p(xd, inverse=inv).cpu().numpy()
        assert p.status() == 0
        ref = orc.c2c_nd(x, dims, inv, batch)
        err = orc.rel_l2(y, ref)
        assert err <= TOL, (dims, batch, inv, err, p.pass_names())
        del y, ref
    del xd
    torch.cuda.empty_cache()
    return x


def test_256cubed_batch8_full(cuda):
    import torch
    from fftgb import api
    from fftgb.plan import Plan
    n, b = 256, 8
    x = _plan_both_directions(cuda, (n, n, n), b, seed=2)
    y, t = api.c2c_3d_ddr_batch(x, n, how_many=b)
    assert t["valid"]
    assert orc.rel_l2(y, orc.c2c_nd(x, (n, n, n), False, b)) <= TOL
    # Parseval per grid, in FP64 over each grid's points
    p = Plan((n, n, n), b)
    xd = torch.from_numpy(x).to(cuda)
    yd = p(xd)
    m = n ** 3
    ex = (xd.view(b, m).abs().double() ** 2).sum(dim=1)
    ey = (yd.view(b, m).abs().double() ** 2).sum(dim=1)
    rel = ((ey / m - ex).abs() / ex).max().item()
    assert rel <= 1e-6, rel


def test_512cubed_full_grid(cuda):
    from fftgb import api
    n = 512
    x = _plan_both_directions(cuda, (n, n, n), 1, seed=3)
    y, t = api.c2c_3d_ddr(x, n)
    assert t["valid"]
    assert orc.rel_l2(y, orc.c2c_nd(x, (n, n, n))) <= TOL


def test_1024sq_batch64_full(cuda):
    from fftgb import api
    n, b = 1024, 64
    x = _plan_both_directions(cuda, (n, n), b, seed=4)
    y, t = api.c2c_2d_bram(x, n, inv=True, how_many=b)
    assert t["valid"]
    assert orc.rel_l2(y, orc.c2c_nd(x, (n, n), True, b)) <= TOL


def test_65536_batch1024_full(cuda):
    from fftgb import api
    n, b = 65536, 1024
    x = _plan_both_directions(cuda, (n,), b, seed=5)
    y, t = api.c2c_1d(x, n, batch=b)
    assert t["valid"]
    ref = orc.c2c_1d(x, n, batch=b)  # bit-reversed within each block
    assert orc.rel_l2(y, ref) <= TOL

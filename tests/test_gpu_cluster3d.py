"""Single-launch 3D transforms of grids up to 2 MiB (k_3d_cluster): one
16-CTA cluster per grid keeps the grid in shared memory across the three
axes.  Every shape with sides in {16, 32, 64}, batches, in place, both
directions and the reference-facing entry points must match the FP64
oracle (rel-L2 <= 2e-6)."""
import itertools

import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6
SHAPES = list(itertools.product((16, 32, 64), repeat=3))  # (nz, ny, nx)


@pytest.mark.parametrize("dims", SHAPES)
def test_cluster_shapes(cuda, monkeypatch, dims):
    import torch
    from fftgb.plan import Plan
    # the default up to 2^15 points; forced above, where it is a tuning choice
    monkeypatch.setenv("FFTGB_CLUSTER", "1")
    batch = 3 if np.prod(dims) <= 32768 else 2
    p = Plan(dims, batch)
    assert p.launches == 1 and p.variant == "cluster", (p.variant, p.pass_names())
    assert p.pass_names()[0] == f"k_3d_cluster<{dims[2]},{dims[1]},{dims[0]}>"
    x = orc.uniform_c64(p.points, seed=int(np.prod(dims)) % 997)
    xd = torch.from_numpy(x).to(cuda)
    for inv in (False, True):
        y = p(xd, inverse=inv).cpu().numpy()
        assert orc.rel_l2(y, orc.c2c_nd(x, dims, inv, batch)) <= TOL, (dims, inv)


def test_cluster_in_place_and_scale(cuda, monkeypatch):
    import torch
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_CLUSTER", "1")
    dims = (64, 64, 64)
    p = Plan(dims, 2)
    assert p.variant == "cluster"
    x = orc.uniform_c64(p.points, seed=5)
    buf = torch.from_numpy(x).to(cuda)
    p(buf, out=buf)
    y = buf.cpu().numpy()
    assert orc.rel_l2(y, orc.c2c_nd(x, dims, False, 2)) <= TOL
    p(buf, inverse=True, scale=1.0 / 64 ** 3, out=buf)
    assert orc.rel_l2(buf.cpu().numpy(), x) <= TOL


def test_cluster_large_batch(cuda, monkeypatch):
    """64 grids of 64^3: many clusters, more than fit the GPU at once."""
    import torch
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_CLUSTER", "1")
    dims, b = (64, 64, 64), 64
    p = Plan(dims, b)
    assert p.variant == "cluster"
    x = orc.uniform_c64(p.points, seed=6)
    y = p(torch.from_numpy(x).to(cuda)).cpu().numpy()
    assert orc.rel_l2(y, orc.c2c_nd(x, dims, False, b)) <= TOL


def test_cluster_default_sizes(cuda):
    """The single launch is the default up to 2^15 points (32^3)."""
    from fftgb.plan import Plan
    assert Plan((32, 32, 32), 1).variant == "cluster"
    assert Plan((16, 32, 64), 4).variant == "cluster"
    assert Plan((64, 64, 64), 1).variant != "cluster"


@pytest.mark.parametrize("n", [16, 32, 64])
def test_abi_3d_bram_and_ddr(cuda, n):
    from fftgb import api
    x = orc.uniform_c64(n ** 3, seed=n)
    for fn in (api.c2c_3d_bram, api.c2c_3d_ddr):
        for inv in (False, True):
            y, t = fn(x, n, inv=inv)
            assert t["valid"]
            assert orc.rel_l2(y, orc.c2c_nd(x, (n, n, n), inv)) <= TOL, (fn, inv)


def test_cluster_unaligned_buffers(cuda):
    """Plain loads and stores: any 8-byte aligned buffer works."""
    import torch
    from fftgb.plan import Plan
    dims = (32, 32, 32)
    p = Plan(dims, 1)
    x = orc.uniform_c64(p.points, seed=9)
    big = torch.zeros(p.points + 1, dtype=torch.complex64, device=cuda)
    big[1:] = torch.from_numpy(x).to(cuda)
    out = torch.zeros_like(big)
    p(big[1:], out=out[1:])
    assert orc.rel_l2(out[1:].cpu().numpy(), orc.c2c_nd(x, dims)) <= TOL

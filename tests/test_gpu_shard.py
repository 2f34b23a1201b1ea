"""Batch sharding on the device: the slices that the ranks of a 2- and
3-process job would transform, run one after another on one GPU, must
reassemble into the unsharded batch transform (rel-L2 <= 2e-6 against the
FP64 oracle, and equal to the unsharded plan's output)."""
import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6


@pytest.mark.parametrize("world", [2, 3])
def test_shards_reassemble(cuda, world):
    import torch
    from fftgb.plan import Plan
    from fftgb.shard import BatchShard
    dims, batch = (64, 64, 64), 5
    n = int(np.prod(dims))
    x = orc.uniform_c64(batch * n, seed=2)
    xd = torch.from_numpy(x).to(cuda)
    full = Plan(dims, batch)(xd)
    parts = []
    for r in range(world):
        sh = BatchShard(dims, batch, world=world, rank=r)
        p = sh.plan()
        if p is None:
            continue
        parts.append(p(sh.local(xd).contiguous()))
    y = torch.cat(parts).cpu().numpy()
    assert torch.equal(torch.from_numpy(y), full.cpu())
    for b in range(batch):
        ref = orc.c2c_nd(x[b * n:(b + 1) * n], dims)
        assert orc.rel_l2(y[b * n:(b + 1) * n], ref) <= TOL

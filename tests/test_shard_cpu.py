"""Batch sharding across processes (CPU: gloo ranks, world size 2 and 3).

Each rank transforms only its own slice of the batch; the FP64 oracle
stands in for the device plan, which cannot run without a GPU.  The
gathered result must equal the unsharded transform exactly, and the
partitions must cover the batch once with balanced loads.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from fftgb import shard
from fftgb import synthetic
from oracle import fft_oracle as orc


def test_batch_partition_covers_once():
    for batch in range(0, 40):
        for world in range(1, 9):
            parts = shard.batch_partition(batch, world)
            assert len(parts) == world
            pos = 0
            for s, c in parts:
                assert s == pos
                pos += c
            assert pos == batch
            counts = [c for _, c in parts]
            assert max(counts) - min(counts) <= 1


def test_batch_partition_rejects_bad_args():
    with pytest.raises(ValueError):
        shard.batch_partition(4, 0)
    with pytest.raises(ValueError):
        shard.batch_partition(-1, 2)
    with pytest.raises(ValueError):
        shard.BatchShard((8, 8, 8), 4, world=2, rank=2)


def test_ragged_partition_balanced():
    shapes, _ = synthetic.ragged_shapes()
    sizes = [int(np.prod(s)) for s in shapes]
    for world in (1, 2, 4, 8):
        parts = shard.ragged_partition(shapes, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(shapes)))
        loads = [sum(sizes[i] for i in p) for p in parts]
        # greedy largest-first: no rank exceeds the mean by more than one grid
        assert max(loads) - sum(loads) / world <= max(sizes)
        assert all(p == sorted(p) for p in parts)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, dims, batch, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sh = shard.BatchShard(dims, batch, world=world, rank=rank)
        n = sh.grid_points
        x = orc.uniform_c64(batch * n, seed=2)
        loc = sh.local(x)
        y = np.concatenate([orc.c2c_nd(loc[i * n:(i + 1) * n], dims).astype(np.complex64)
                            for i in range(sh.count)]) if sh.count else np.zeros(0, np.complex64)
        full = shard.gather(torch.from_numpy(y), sh)
        if rank == 0:
            q.put(full.numpy())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,batch", [(2, 5), (3, 2)])
def test_gloo_sharded_batch_matches_unsharded(world, batch):
    dims = (8, 16, 4)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, dims, batch, q))
             for r in range(world)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    n = int(np.prod(dims))
    x = orc.uniform_c64(batch * n, seed=2)
    ref = np.concatenate([orc.c2c_nd(x[i * n:(i + 1) * n], dims).astype(np.complex64)
                          for i in range(batch)])
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)


def test_ragged_shapes_pinned():
    import json
    path = os.path.join(os.path.dirname(__file__), "golden", "ragged48_shapes.json")
    with open(path) as f:
        pin = json.load(f)
    shapes, seed = synthetic.ragged_shapes()
    assert seed == pin["seed"]
    assert [list(s) for s in shapes] == pin["shapes"]
    assert sum(int(np.prod(s)) for s in shapes) * 8 == pin["bytes"]
    assert abs(pin["bytes"] - 2 * 2 ** 30) <= 0.1 * 2 * 2 ** 30

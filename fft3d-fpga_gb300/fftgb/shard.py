"""Batch sharding across processes, one GPU per process.

Every transform of a batched or ragged call is independent, so N processes
split the batch and run with no collective on the data path: rank r
transforms its own contiguous slice of the batch (or its own subset of the
ragged grids) on its own GPU.  The reference runs one FPGA per process and
has no multi-device path (api/src/fftfpga.c:37-142 selects one device);
this module is the partitioner a multi-GPU caller adds on top.

An optional host-side gather (``gather``) uses whatever process group the
caller initialised (gloo on CPU, NCCL on GPUs); it is not part of a step.
"""
from __future__ import annotations

import os
from dataclasses import dataclass


def world_from_env() -> tuple[int, int]:
    """(world_size, rank) from the torchrun environment (1, 0 without)."""
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))


def batch_partition(batch: int, world: int) -> list[tuple[int, int]]:
    """Contiguous (start, count) per rank; counts differ by at most one and
    the first ``batch % world`` ranks take the extra transform."""
    if batch < 0 or world < 1:
        raise ValueError("batch >= 0 and world >= 1 required")
    q, r = divmod(batch, world)
    out, start = [], 0
    for k in range(world):
        c = q + (1 if k < r else 0)
        out.append((start, c))
        start += c
    return out


def ragged_partition(shapes, world: int) -> list[list[int]]:
    """Grid indices per rank, balancing points (the HBM traffic of a grid is
    proportional to its points): largest grid first onto the least loaded
    rank, ties to the lower rank.  Each rank's list is in ascending order so
    its grids keep their order in the packed buffer."""
    if world < 1:
        raise ValueError("world >= 1 required")
    sizes = []
    for i, s in enumerate(shapes):
        n = 1
        for d in s:
            n *= int(d)
        sizes.append((n, i))
    load = [0] * world
    owner = [[] for _ in range(world)]
    for n, i in sorted(sizes, key=lambda t: (-t[0], t[1])):
        k = min(range(world), key=lambda r: (load[r], r))
        load[k] += n
        owner[k].append(i)
    return [sorted(o) for o in owner]


@dataclass
class BatchShard:
    """This rank's share of a batch of ``batch`` grids of ``dims`` points each
    (dims slowest first)."""
    dims: tuple
    batch: int
    world: int = 1
    rank: int = 0

    def __post_init__(self):
        self.dims = tuple(int(d) for d in self.dims)
        if not 0 <= self.rank < self.world:
            raise ValueError("rank out of range")
        self.start, self.count = batch_partition(self.batch, self.world)[self.rank]
        self.grid_points = 1
        for d in self.dims:
            self.grid_points *= d

    @property
    def point_range(self) -> tuple[int, int]:
        """[begin, end) of this rank's points in the packed batch."""
        return self.start * self.grid_points, (self.start + self.count) * self.grid_points

    def local(self, x):
        """This rank's slice of a packed batch (a view for numpy and torch)."""
        a, b = self.point_range
        return x[a:b]

    def plan(self, **kw):
        """A device plan for this rank's transforms (None if it has none)."""
        if self.count == 0:
            return None
        from .plan import Plan
        return Plan(self.dims, self.count, **kw)


def gather(local, shard: BatchShard, group=None):
    """Concatenate every rank's slice in batch order on every rank (host
    side, through torch.distributed.all_gather; slices may differ in size)."""
    import torch
    import torch.distributed as dist

    parts = batch_partition(shard.batch, shard.world)
    flat = local.reshape(-1)
    cplx = flat.is_complex()
    if cplx:  # gloo moves real tensors only
        flat = torch.view_as_real(flat).reshape(-1)
    w = 2 if cplx else 1
    maxn = max(c for _, c in parts) * shard.grid_points * w
    buf = torch.zeros(maxn, dtype=flat.dtype, device=flat.device)
    buf[:flat.numel()] = flat
    bufs = [torch.empty_like(buf) for _ in range(shard.world)]
    dist.all_gather(bufs, buf, group=group)
    out = torch.cat([bufs[k][:parts[k][1] * shard.grid_points * w]
                     for k in range(shard.world)])
    return torch.view_as_complex(out.reshape(-1, 2)) if cplx else out

"""Ragged batches of 3D grids with independent shapes (powers of two in the
persistent kernel, other lengths as plans of their own).

The persistent form (one kernel launch for the whole batch) and the
graph-of-plans form must both match the FP64 oracle grid by grid
(rel-L2 <= 2e-6).  The 48-grid workload of about 2 GiB is checked on a
subset of grids against the oracle and on all grids by a round trip.
"""
import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _check(cuda, shapes, expect_launches=None, seed=8):
    import torch
    from fftgb.plan import RaggedPlan
    rp = RaggedPlan(shapes)
    if expect_launches is not None:
        assert rp.launches == expect_launches
    x = orc.uniform_c64(rp.points, seed=seed)
    xd = torch.from_numpy(x).to(cuda)
    for inv in (False, True):
        y = rp(xd, inverse=inv).cpu().numpy()
        assert rp.status() == 0
        off = 0
        for s in shapes:
            n = int(np.prod(s))
            ref = orc.c2c_nd(x[off:off + n], s, inv)
            assert orc.rel_l2(y[off:off + n], ref) <= TOL, (s, inv)
            off += n


def test_ragged_persistent(cuda):
    rng = np.random.default_rng(3)
    shapes = [tuple(int(v) for v in rng.choice([16, 32, 64, 128], 3)) for _ in range(9)]
    shapes.append((64, 128, 256))
    _check(cuda, shapes, expect_launches=1)


# every two-pass tile combination: pass A (nx, rows per tile) and pass B
# (nz, radix R), plus shapes that fall back to one pass per axis
FUSED_SHAPES = [
    (16, 64, 32), (32, 32, 32), (64, 128, 32), (32, 256, 32), (32, 32, 64),
    (64, 64, 64), (64, 256, 64), (64, 32, 128), (32, 128, 128), (128, 256, 128),
    (64, 128, 256), (32, 256, 256), (64, 256, 256), (128, 64, 256), (256, 128, 256),
    (256, 64, 256), (128, 256, 256), (32, 128, 256), (256, 256, 256),
    (32, 512, 32), (32, 256, 64), (16, 16, 16),
]


def test_ragged_two_pass_tiles(cuda, monkeypatch):
    # every shape in the work list (256 x 256 x 256 would otherwise run as a
    # grouped uniform pass pair)
    monkeypatch.setenv("FFTGB_RAGGED_NO_GROUP", "1")
    _check(cuda, FUSED_SHAPES, expect_launches=1, seed=11)


GROUPED_SHAPES = [(256, 256, 256), (64, 64, 64), (256, 256, 128), (32, 128, 256),
                  (256, 256, 256), (256, 256, 128), (16, 32, 64), (256, 256, 128)]


def test_ragged_grouped_uniform_passes(cuda, monkeypatch):
    """Grids of 256 x 256 x {128, 256} leave the work list and run as
    grouped launches of the uniform TMA-fed pass pair (per-grid tensor
    maps), the rest in the persistent kernel: 1 + 2 + 2 launches.  Every
    grid against the oracle, both directions, and against the plan that
    keeps every grid in the work list."""
    import torch
    from fftgb.plan import RaggedPlan
    _check(cuda, GROUPED_SHAPES, expect_launches=5, seed=13)
    x = orc.uniform_c64(RaggedPlan(GROUPED_SHAPES).points, seed=14)
    xd = torch.from_numpy(x).to(cuda)
    y = RaggedPlan(GROUPED_SHAPES)(xd).cpu().numpy()
    monkeypatch.setenv("FFTGB_RAGGED_NO_GROUP", "1")
    rq = RaggedPlan(GROUPED_SHAPES)
    assert rq.launches == 1
    assert orc.rel_l2(y, rq(xd).cpu().numpy()) <= TOL


def test_ragged_grouped_unaligned_and_many(cuda):
    """Buffers only 8-byte aligned: the grouped grids run grid by grid on
    the one-tile kernels (same transform).  A group of 15 grids runs as two
    launches of each pass (14 + 1 grids) and no work list."""
    import torch
    from fftgb.plan import RaggedPlan
    rp = RaggedPlan(GROUPED_SHAPES)
    x = orc.uniform_c64(rp.points, seed=15)
    big = torch.zeros(rp.points + 1, dtype=torch.complex64, device=cuda)
    big[1:] = torch.from_numpy(x).to(cuda)
    out = torch.zeros_like(big)
    rp(big[1:], out=out[1:])
    assert rp.status() == 0
    y = out[1:].cpu().numpy()
    off = 0
    for s in GROUPED_SHAPES:
        n = int(np.prod(s))
        assert orc.rel_l2(y[off:off + n], orc.c2c_nd(x[off:off + n], s)) <= TOL, s
        off += n
    del big, out
    shapes = [(256, 256, 128)] * 15
    rp = RaggedPlan(shapes)
    assert rp.launches == 4
    g = torch.Generator(device=cuda).manual_seed(16)
    xd = torch.view_as_complex((torch.rand(rp.points, 2, device=cuda, generator=g) * 2 - 1).contiguous())
    yd = rp(xd)
    assert rp.status() == 0
    n = 256 * 256 * 128
    for i in (0, 13, 14):
        ref = orc.c2c_nd(xd[i * n:(i + 1) * n].cpu().numpy(), shapes[i])
        assert orc.rel_l2(yd[i * n:(i + 1) * n].cpu().numpy(), ref) <= TOL, i
    ex = (xd.view(15, n).abs().double() ** 2).sum(dim=1)
    ey = (yd.view(15, n).abs().double() ** 2).sum(dim=1)
    assert ((ey / n - ex).abs() / ex).max().item() <= 1e-6


def test_ragged_axis_passes(cuda, monkeypatch):
    monkeypatch.setenv("FFTGB_RAGGED_AXES", "1")
    _check(cuda, FUSED_SHAPES[:12], expect_launches=1, seed=12)


def test_ragged_graph_form(cuda, monkeypatch):
    monkeypatch.setenv("FFTGB_RAGGED_GRAPH", "1")
    rng = np.random.default_rng(4)
    shapes = [tuple(int(v) for v in rng.choice([16, 32, 64], 3)) for _ in range(5)]
    _check(cuda, shapes)


def test_ragged_small_axes_fall_back(cuda):
    # axis lengths 2..8 are outside the persistent kernel's set
    shapes = [(8, 16, 32), (4, 4, 4), (32, 2, 16)]
    _check(cuda, shapes)


def test_ragged_48_grids_2gib(cuda):
    import torch
    from fftgb import synthetic
    from fftgb.plan import RaggedPlan
    shapes, _ = synthetic.ragged_shapes()
    assert len(shapes) == 48
    rp = RaggedPlan(shapes)
    # the persistent kernel, and a grouped pass pair for the 256^3 grids and
    # one for the 256 x 256 x 128 grids
    assert rp.launches == 5
    assert abs(rp.points * 8 - 2 * 2 ** 30) <= 0.1 * 2 * 2 ** 30
    g = torch.Generator(device=cuda).manual_seed(8)
    x = torch.view_as_complex((torch.rand(rp.points, 2, device=cuda, generator=g) * 2 - 1).contiguous())
    y = rp(x)
    z = rp(y, inverse=True)
    assert rp.status() == 0
    offs = np.cumsum([0] + [int(np.prod(s)) for s in shapes])
    # every grid: round trip (the inverse is unnormalised)
    for i, s in enumerate(shapes):
        n = int(np.prod(s))
        a, b = int(offs[i]), int(offs[i + 1])
        err = ((z[a:b] / n - x[a:b]).abs() ** 2).double().sum().sqrt() / \
            (x[a:b].abs() ** 2).double().sum().sqrt()
        assert err.item() <= 2 * TOL, s
        # Parseval: sum |X|^2 = n sum |x|^2 for every grid
        ex = (x[a:b].abs().double() ** 2).sum()
        ey = (y[a:b].abs().double() ** 2).sum()
        assert abs(ey.item() / n - ex.item()) <= 1e-6 * ex.item(), s
    # a few grids of different shapes against the oracle
    for i in sorted(set([0, 7, 23, 47])):
        a, b = int(offs[i]), int(offs[i + 1])
        ref = orc.c2c_nd(x[a:b].cpu().numpy(), shapes[i])
        assert orc.rel_l2(y[a:b].cpu().numpy(), ref) <= TOL, shapes[i]


def test_ragged_survives_final_and_reinit(cuda, tmp_path):
    """fpga_final releases the shared twiddle tables; a ragged plan made
    before it re-captures its launch when it runs again (stale table
    pointers would give wrong results), its grouped passes included."""
    import torch
    from fftgb import api
    from fftgb.plan import RaggedPlan
    shapes = [(32, 64, 128), (64, 64, 64), (16, 32, 32), (256, 256, 128)]
    rp = RaggedPlan(shapes)
    assert rp.launches == 3
    x = orc.uniform_c64(rp.points, seed=5)
    xd = torch.from_numpy(x).to(cuda)
    y0 = rp(xd).cpu().numpy()
    f = tmp_path / "p.json"
    f.write_text("{}")
    assert api.initialize("NVIDIA CUDA", str(f)) == 0
    api.final()
    torch.cuda.synchronize()
    y1 = rp(xd).cpu().numpy()
    assert rp.status() == 0
    off = 0
    for s in shapes:
        n = int(np.prod(s))
        ref = orc.c2c_nd(x[off:off + n], s)
        assert orc.rel_l2(y1[off:off + n], ref) <= TOL
        off += n
    assert np.array_equal(y0, y1)


@pytest.mark.parametrize("shapes,persistent", [
    # power-of-two grids in the persistent kernel, the others as plans of their own
    ([(96, 96, 96), (64, 64, 64), (30, 48, 100), (128, 128, 128), (45, 27, 64), (16, 32, 64)],
     True),
    # a grouped 256^3 grid beside mixed-radix and Bluestein grids
    ([(256, 256, 256), (100, 100, 100), (7, 9, 32)], True),
    # no power-of-two grid at all
    ([(96, 96, 96), (120, 120, 120), (3, 5, 6)], False),
])
def test_ragged_not_power_of_two(cuda, shapes, persistent):
    """Grids whose sides are not all powers of two join the batch as plans of
    their own (mixed-radix or Bluestein) in the same graph."""
    from fftgb.plan import Plan
    extra = sum(len(Plan(s, 1).pass_names()) for s in shapes
                if any(v & (v - 1) for v in s))
    import torch
    from fftgb.plan import RaggedPlan
    rp = RaggedPlan(shapes)
    assert rp.launches >= extra + (1 if persistent else 0), rp.launches
    x = orc.uniform_c64(rp.points, seed=21)
    xd = torch.from_numpy(x).to(cuda)
    for inv in (False, True):
        y = rp(xd, inverse=inv).cpu().numpy()
        assert rp.status() == 0
        off = 0
        for s in shapes:
            n = int(np.prod(s))
            ref = orc.c2c_nd(x[off:off + n], s, inv)
            assert orc.rel_l2(y[off:off + n], ref) <= TOL, (s, inv)
            off += n

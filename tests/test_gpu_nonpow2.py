"""Axis lengths that are not powers of two (no reference counterpart, the
reference takes powers of two only).  Lengths 2^a 3^b 5^c up to 8192 take
the mixed-radix line kernel (`k_mix`, Stockham stages of radix 16, 15, 12,
10, 9, 8, 6, 5, 4, 3 and 2),
any other length up to 2048 Bluestein's algorithm (`k_blue`); FFTGB_NO_MIX=1
sends the smooth lengths to Bluestein as well, so both kernels are checked
on the same sizes.  1D, 2D, 3D and mixed grids against the FP64 oracle, both
directions, scaling, in place, and the rejected cases.  Tolerances: rel-L2
<= 1e-6 for the mixed-radix plans (FP64 twiddle table, log n stages),
<= 2e-6 for Bluestein (two M-point transforms, M >= 2n - 1)."""
import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL_BLUE = 2e-6
TOL_MIX = 1e-6


def _smooth(n):
    for f in (2, 3, 5):
        while n % f == 0:
            n //= f
    return n == 1


def _run(cuda, dims, batch, inplace=False, scale=1.0, variant=None):
    import torch
    from fftgb.plan import Plan
    p = Plan(dims, batch)
    if variant is None:
        variant = "mixed" if all(_smooth(d) for d in dims) else "bluestein"
    assert p.variant == variant, (dims, p.variant, p.pass_names())
    tol = TOL_MIX if variant.startswith("mixed") else TOL_BLUE
    x = orc.uniform_c64(p.points, seed=sum(dims) + batch)
    for inv in (False, True):
        xd = torch.from_numpy(x).to(cuda)
        y = p(xd, inverse=inv, scale=scale, out=xd if inplace else None).cpu().numpy()
        ref = scale * orc.c2c_nd(x, dims, inv, batch)
        assert orc.rel_l2(y, ref) <= tol, (dims, inv, p.pass_names(), orc.rel_l2(y, ref))
    return p


@pytest.mark.parametrize("n", [7, 11, 2047, 1022, 11 * 13, 2 * 1021])
def test_1d_bluestein(cuda, n):
    p = _run(cuda, (n,), 3)
    assert p.pass_names()[0].startswith("k_blue"), p.pass_names()


@pytest.mark.parametrize("n", [6, 12, 100, 125, 243, 1000, 1536])
def test_1d_smooth_through_bluestein(cuda, monkeypatch, n):
    monkeypatch.setenv("FFTGB_NO_MIX", "1")
    p = _run(cuda, (n,), 3, variant="bluestein")
    assert p.pass_names()[0].startswith("k_blue"), p.pass_names()


@pytest.mark.parametrize("n", [3, 5, 6, 9, 10, 12, 15, 18, 20, 24, 25, 27, 30, 45, 48, 60, 72,
                               80, 96, 100, 120, 125, 160, 240, 243, 250, 320, 384, 480, 500,
                               640, 729, 768, 960, 1000, 1080, 1200, 1536, 2000, 2187, 2400,
                               3000, 3072, 3125, 3840, 4000, 4800, 6000, 6144, 6561, 7680, 8000])
def test_1d_mixed(cuda, n):
    p = _run(cuda, (n,), 3)
    names = p.pass_names()
    if n <= 4096:
        assert len(names) == 1 and names[0].startswith(f"k_mix<n={n},"), names
    else:  # the four-step: twiddled columns, then transposed rows
        assert len(names) == 2 and names[0].endswith(",tw>") and names[1].endswith(",tr>"), names


@pytest.mark.parametrize("n,batch", [(10000, 3), (12000, 2), (4500, 5), (100000, 2),
                                     (1000000, 1), (3 * 2 ** 20, 1), (16000000, 1),
                                     (5 ** 7, 1)])
def test_1d_mixed_fourstep(cuda, n, batch):
    """1D lengths 2^a 3^b 5^c above 4096 (up to 2^24): n = n1 * n2, the
    n2-point columns times W_n^(j1 k2), then the n1-point rows stored
    transposed."""
    p = _run(cuda, (n,), batch)
    names = p.pass_names()
    assert len(names) == 2 and names[0].endswith(",tw>") and names[1].endswith(",tr>"), names
    n2 = int(names[0].split("n=")[1].split(",")[0])
    n1 = int(names[1].split("n=")[1].split(",")[0])
    assert n1 * n2 == n


@pytest.mark.parametrize("n,batch", [(96, 1), (96, 17), (1000, 5), (240, 33), (6000, 2),
                                     (15, 1000), (3, 4097)])
def test_1d_mixed_line_counts(cuda, n, batch):
    """Line counts that fill no whole CTA (lines per CTA are a power of two)."""
    _run(cuda, (n,), batch)


def test_mixed_radices_in_pass_names(cuda):
    """The fewest stages (radix 16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2) that
    fit the 256-thread CTAs, else the 512-thread ones."""
    from fftgb.plan import Plan
    for n, rad in [(240, "16x15"), (1000, "10x10x10"), (96, "16x6"), (2187, "9x9x9x3"),
                   (4000, "16x5x5x5x2"), (6, "6"), (243, "9x9x3"), (3000, "15x8x5x5")]:
        assert Plan((n,), 1).pass_names() == [f"k_mix<n={n},{rad}>"], n
    # 2D / 3D axes above 4096 stay one pass (the four-step is for 1D plans)
    assert Plan((2, 6561), 1).pass_names()[0] == "k_mix<n=6561,9x9x9x9>"


@pytest.mark.parametrize("n,rad", [(240, "16x5x3"), (1000, "8x5x5x5"), (96, "16x3x2"),
                                   (2187, "3x3x3x3x3x3x3"), (4000, "16x5x5x5x2"), (6, "3x2"),
                                   (250, "5x5x5x2"), (3000, "8x5x5x5x3"), (64 * 3, "16x4x3")])
def test_mixed_simple_radices(cuda, monkeypatch, n, rad):
    """FFTGB_MIX_SIMPLE=1: stages of radix 16, 8, 4, 2, 5 and 3 only (every
    radix kernel body on its own)."""
    monkeypatch.setenv("FFTGB_MIX_SIMPLE", "1")
    p = _run(cuda, (n,), 3, variant="mixed:simple")
    assert p.pass_names() == [f"k_mix<n={n},{rad}>"], p.pass_names()
    _run(cuda, (n, 4), 2, variant="mixed:simple")


@pytest.mark.parametrize("dims,batch", [((96, 96, 96), 1), ((243, 30), 2), ((1000,), 3),
                                        ((100, 240), 2), ((6, 4000), 1), ((15, 3000), 2)])
def test_generic_kernel(cuda, monkeypatch, dims, batch):
    """FFTGB_MIX_GENERIC=1: the kernel that holds every radix, instead of the
    two- and three-stage instantiations (k_mix2 / k_mix3) the plans launch."""
    monkeypatch.setenv("FFTGB_MIX_GENERIC", "1")
    _run(cuda, dims, batch)


@pytest.mark.parametrize("dims,batch", [
    ((60, 100), 2), ((1000, 48), 1), ((100, 64), 3), ((64, 100), 2), ((7, 9), 5),
    ((3, 1000), 2), ((1000, 3), 2), ((5, 7), 3), ((6000, 4), 1), ((4, 6000), 1),
    ((120, 7), 2),
])
def test_2d(cuda, dims, batch):
    _run(cuda, dims, batch)


@pytest.mark.parametrize("dims,batch", [
    ((27, 45, 64), 1), ((16, 12, 10), 3), ((125, 125, 125), 1), ((96, 96, 96), 1),
    ((64, 64, 3), 2), ((100, 100, 100), 1), ((120, 120, 120), 2), ((240, 240, 240), 1),
    ((7, 96, 5), 2), ((2, 3, 1000), 3),
])
def test_3d(cuda, dims, batch):
    p = _run(cuda, dims, batch)
    names = p.pass_names()
    assert any(n.startswith("k_mix") or n.startswith("k_blue") for n in names), names


@pytest.mark.parametrize("dims,batch", [((96, 96, 96), 2), ((27, 45, 64), 1)])
def test_3d_bluestein_and_mixed_agree(cuda, monkeypatch, dims, batch):
    """The same smooth grid through both kernels: each against the oracle,
    and the two within their combined tolerance of each other."""
    import torch
    from fftgb.plan import Plan
    x = orc.uniform_c64(int(np.prod(dims)) * batch, seed=5)
    xd = torch.from_numpy(x).to(cuda)
    ym = Plan(dims, batch)(xd).cpu().numpy()
    monkeypatch.setenv("FFTGB_NO_MIX", "1")
    pb = Plan(dims, batch)
    assert pb.variant == "bluestein"
    yb = pb(xd).cpu().numpy()
    ref = orc.c2c_nd(x, dims, False, batch)
    assert orc.rel_l2(ym, ref) <= TOL_MIX
    assert orc.rel_l2(yb, ref) <= TOL_BLUE
    assert orc.rel_l2(ym, yb) <= TOL_MIX + TOL_BLUE


def test_scale_and_in_place(cuda):
    _run(cuda, (30, 50), 2, inplace=True, scale=0.125)
    _run(cuda, (7, 50), 2, inplace=True, scale=0.5)
    _run(cuda, (1000,), 7, inplace=True, scale=1.0 / 1000)


def test_mixed_round_trip(cuda):
    import torch
    from fftgb.plan import Plan
    for dims, batch in [((6000,), 2), ((96, 96, 96), 1), ((3, 5, 15), 4)]:
        p = Plan(dims, batch)
        x = orc.uniform_c64(p.points, seed=3)
        xd = torch.from_numpy(x).to(cuda)
        z = p(p(xd), inverse=True, scale=1.0 / int(np.prod(dims))).cpu().numpy()
        assert orc.rel_l2(z, x) <= 2 * TOL_MIX, dims


def test_rejected(cuda):
    from fftgb import FFTGBError
    from fftgb.plan import Plan
    for args, kw in [(((2049,), 1), {}), (((100,), 1), {"order": "bitrev"}),
                     (((100,), 1), {"precision": "tc_fp16"}), (((8192, 3), 1), {}),
                     (((20000000,), 1), {}), (((3 * 2741,), 1), {}), (((10000, 2), 1), {})]:
        with pytest.raises(FFTGBError):
            Plan(*args, **kw)


def test_autotune_and_tuning_cache(cuda, lib, tmp_path):
    """The non-power-of-two plans' decompositions are autotuner candidates:
    "mixed" (composite radices), "mixed:simple" (radix 16/8/4/2/5/3 only)
    and "bluestein" (axes up to 2048).  A tuning-cache entry picks one, the
    tuner times them and keeps a correct plan, and dropping the cache gives
    the default again."""
    import torch
    from fftgb.plan import Plan
    cache = tmp_path / "tune.json"
    cache.write_text('{"3000,1,1,2,0": "mixed:simple", "96,96,96,1,0": "bluestein"}')
    assert lib.fftgb_tune_cache(str(cache).encode()) == 0
    try:
        p = Plan((3000,), 2)
        assert p.variant == "mixed:simple", p.variant
        assert p.pass_names() == ["k_mix<n=3000,8x5x5x5x3>"], p.pass_names()
        q = Plan((96, 96, 96), 1)
        assert q.variant == "bluestein" and q.pass_names()[0].startswith("k_blue"), q.pass_names()
        for plan, dims, batch, names in [(p, (3000,), 2, ("mixed=", "mixed:simple=")),
                                         (q, (96, 96, 96), 1,
                                          ("mixed=", "mixed:simple=", "bluestein="))]:
            report = plan.autotune(reps=2)
            for nm in names:
                assert nm in report, report
            x = orc.uniform_c64(plan.points, seed=12)
            xd = torch.from_numpy(x).to(cuda)
            for inv in (False, True):
                y = plan(xd, inverse=inv).cpu().numpy()
                ref = orc.c2c_nd(x, dims, inv, batch)
                tol = TOL_MIX if plan.variant.startswith("mixed") else TOL_BLUE
                assert orc.rel_l2(y, ref) <= tol, (plan.variant, inv)
    finally:
        lib.fftgb_tune_cache(b"")
    assert Plan((3000,), 2).variant == "mixed"
    assert Plan((96, 96, 96), 1).pass_names() == ["k_mix<n=96,16x6>"] * 3


@pytest.mark.parametrize("dims,batch", [((96, 100, 30), 2), ((45, 27, 64), 1), ((5, 7, 9), 3),
                                        ((64, 64, 96), 1)])
def test_poisson_filter(cuda, dims, batch):
    """The Poisson filter G = 1/|k|^2 (k = n fftfreq(n), odd sides included)
    on non-power-of-two plans: one element-wise pass after the transform,
    forward and adjoint, against G . FFT in FP64."""
    import torch
    from fftgb.plan import Plan
    p = Plan(dims, batch)
    x = orc.uniform_c64(p.points, seed=33)
    xd = torch.from_numpy(x).to(cuda)
    ks = np.meshgrid(*[np.fft.fftfreq(d, d=1.0 / d) for d in dims], indexing="ij")
    k2 = sum(k ** 2 for k in ks)
    G = np.tile(np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0).reshape(-1), batch)
    tol = TOL_MIX if p.variant.startswith("mixed") else TOL_BLUE
    y = p.execute(xd, filter="poisson").cpu().numpy()
    assert orc.rel_l2(y, G * orc.c2c_nd(x, dims, False, batch)) <= tol
    ya = p.execute(xd, adjoint=True, filter="poisson", scale=0.5).cpu().numpy()
    assert orc.rel_l2(ya, 0.5 * G * orc.c2c_nd(x, dims, True, batch)) <= tol


@pytest.mark.parametrize("dims,batch", [((96, 96, 96), 1), ((240,), 7), ((100, 30), 3),
                                        ((6, 8, 960), 1)])
def test_mixed_unaligned_buffers(cuda, dims, batch):
    """Buffers only 8-byte aligned (one complex64 past a 256-byte boundary),
    out of place and in place."""
    import torch
    from fftgb.plan import Plan
    p = Plan(dims, batch)
    x = orc.uniform_c64(p.points, seed=44)
    ref = orc.c2c_nd(x, dims, False, batch)
    big = torch.zeros(p.points + 1, dtype=torch.complex64, device=cuda)
    big[1:] = torch.from_numpy(x).to(cuda)
    out = torch.zeros_like(big)
    p(big[1:], out=out[1:])
    assert orc.rel_l2(out[1:].cpu().numpy(), ref) <= TOL_MIX
    p(big[1:], out=big[1:])
    assert orc.rel_l2(big[1:].cpu().numpy(), ref) <= TOL_MIX

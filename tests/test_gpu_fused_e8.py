"""The one-tile fused passes with 8 points per thread (variant bit 8:
"fused:64:32:p8", `k_xy<64,64,e8>` + `k_rz<64,1,32,e8>`), the plan of the
latency-bound single 64^3 grid.  Every case against the FP64 oracle
(rel-L2 <= 2e-6): both directions, scaled round trip, in place, buffers only
8-byte aligned, the fused Poisson filter and the adjoint."""
import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _plan(monkeypatch, dims, batch):
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_FUSED_NJ", "64")
    monkeypatch.setenv("FFTGB_FUSED_X", "32")
    monkeypatch.setenv("FFTGB_FUSED_PIPE", "8")
    p = Plan(dims, batch)
    assert p.pass_names() == ["k_xy<64,64,e8>", "k_rz<64,1,32,e8>"], p.pass_names()
    return p


@pytest.mark.parametrize("batch", [1, 3])
def test_e8_pair_directions_and_round_trip(cuda, monkeypatch, batch):
    import torch
    dims = (64, 64, 64)
    p = _plan(monkeypatch, dims, batch)
    x = orc.uniform_c64(p.points, seed=80 + batch)
    xd = torch.from_numpy(x).to(cuda)
    for inv in (False, True):
        y = p(xd, inverse=inv).cpu().numpy()
        assert orc.rel_l2(y, orc.c2c_nd(x, dims, inv, batch)) <= TOL, inv
    n = int(np.prod(dims))
    z = p(p(xd), inverse=True, scale=1.0 / n).cpu().numpy()
    assert orc.rel_l2(z, x) <= 2 * TOL
    # in place (pass B reads and writes the same rows; R = 1)
    buf = xd.clone()
    p(buf, out=buf)
    assert orc.rel_l2(buf.cpu().numpy(), orc.c2c_nd(x, dims, False, batch)) <= TOL


def test_e8_pair_unaligned_filter_adjoint(cuda, monkeypatch):
    import torch
    dims, batch = (64, 64, 64), 2
    p = _plan(monkeypatch, dims, batch)
    x = orc.uniform_c64(p.points, seed=90)
    xd = torch.from_numpy(x).to(cuda)
    ref = orc.c2c_nd(x, dims, False, batch)
    big = torch.zeros(p.points + 1, dtype=torch.complex64, device=cuda)
    big[1:] = xd
    out = torch.zeros_like(big)
    p(big[1:], out=out[1:])
    assert orc.rel_l2(out[1:].cpu().numpy(), ref) <= TOL
    ks = np.meshgrid(*[np.fft.fftfreq(d, d=1.0 / d) for d in dims], indexing="ij")
    k2 = sum(k ** 2 for k in ks)
    G = np.tile(np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0).reshape(-1), batch)
    yf = p.execute(xd, filter="poisson").cpu().numpy()
    assert orc.rel_l2(yf, G * ref) <= TOL
    ya = p.execute(xd, adjoint=True, scale=0.25).cpu().numpy()
    assert orc.rel_l2(ya, 0.25 * orc.c2c_nd(x, dims, True, batch)) <= TOL


def test_e8_variant_string_round_trips_through_the_tuning_cache(cuda, lib, tmp_path):
    """A tuning-cache entry naming an 8-points-per-thread plan gives that
    plan, the autotuner lists the pair among the 64^3 candidates, and
    dropping the cache (fftgb_tune_cache(NULL)) forgets the entries: the
    next plan of the shape takes the measured default again."""
    import torch
    from fftgb.plan import Plan
    cache = tmp_path / "tune.json"
    cache.write_text('{"64,64,64,2,0": "fused:64:64:p8"}')
    assert lib.fftgb_tune_cache(str(cache).encode()) == 0
    try:
        p = Plan((64, 64, 64), 2)
        assert p.variant == "fused:64:64:p8", p.variant
        assert p.pass_names() == ["k_xy<64,64,e8>", "k_rz<64,1,64>"], p.pass_names()
        x = orc.uniform_c64(p.points, seed=91)
        y = p(torch.from_numpy(x).to(cuda)).cpu().numpy()
        assert orc.rel_l2(y, orc.c2c_nd(x, (64, 64, 64), False, 2)) <= TOL
        report = p.autotune(reps=2)
        assert "fused:64:32:p8=" in report, report
    finally:
        lib.fftgb_tune_cache(b"")
    assert Plan((64, 64, 64), 2).variant == "fused:64:32:p8"

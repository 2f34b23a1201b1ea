"""Per-axis 3D plans with the y-blocked intermediate layout (variant
"axis:b8"): pass 1 (x) writes rows to [b][ny/8][nz][8][nx], pass 2 (z) is a
column pass of stride 8*nx, pass 3 (y) reads 8-row blocks by 5D tensor
copies and writes the natural layout.  The default where a z-plane is 2 MiB
or more and the y axis has a TMA column pass; the plan needs its work
buffer and cannot run in place.  Every case against the FP64 oracle
(rel-L2 <= 2e-6) and against the natural-layout plan."""
import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6
SHAPES = [((4, 512, 512), 1), ((2, 512, 512), 3), ((8, 256, 1024), 1),
          ((16, 128, 2048), 1), ((64, 256, 1024), 1)]


@pytest.mark.parametrize("dims,batch", SHAPES)
def test_blocked_plan(cuda, dims, batch):
    import torch
    from fftgb.plan import Plan
    p = Plan(dims, batch)
    assert p.variant == "axis:b8", p.variant
    names = p.pass_names()
    assert names[0].startswith("k_rows") and names[2].startswith("k_cols_tma"), names
    x = orc.uniform_c64(p.points, seed=sum(dims) + batch)
    xd = torch.from_numpy(x).to(cuda)
    n = int(np.prod(dims))
    for inv in (False, True):
        y = p(xd, inverse=inv).cpu().numpy()
        assert orc.rel_l2(y, orc.c2c_nd(x, dims, inv, batch)) <= TOL, (names, inv)
    z = p(p(xd), inverse=True, scale=1.0 / n).cpu().numpy()
    assert orc.rel_l2(z, x) <= 2 * TOL


def test_blocked_matches_natural_and_edges(cuda, monkeypatch):
    import torch
    from fftgb import _lib
    from fftgb.plan import Plan
    dims, batch = (4, 512, 512), 2
    p = Plan(dims, batch)
    assert p.variant == "axis:b8"
    monkeypatch.setenv("FFTGB_NO_BLK", "1")
    q = Plan(dims, batch)
    monkeypatch.delenv("FFTGB_NO_BLK")
    assert q.variant != "axis:b8"
    x = orc.uniform_c64(p.points, seed=3)
    xd = torch.from_numpy(x).to(cuda)
    assert orc.rel_l2(p(xd).cpu().numpy(), q(xd).cpu().numpy()) <= 1e-6
    # in place is refused (pass 1 remaps rows)
    buf = xd.clone()
    with pytest.raises(_lib.FFTGBError):
        p(buf, out=buf)
    # input and output only 8-byte aligned (per-thread stores in pass 3)
    ref = orc.c2c_nd(x, dims, False, batch)
    big = torch.zeros(p.points + 1, dtype=torch.complex64, device=cuda)
    big[1:] = xd
    out = torch.zeros_like(big)
    p(big[1:], out=out[1:])
    assert orc.rel_l2(out[1:].cpu().numpy(), ref) <= TOL
    # adjoint and the Poisson filter on the blocked plan
    ya = p.execute(xd, adjoint=True, scale=0.5).cpu().numpy()
    assert orc.rel_l2(ya, 0.5 * orc.c2c_nd(x, dims, True, batch)) <= TOL


def test_blocked_variant_autotune_and_cache(cuda, lib, tmp_path):
    """The autotuner times the y-blocked plan beside the natural per-axis
    plan; whichever it keeps is recorded in the tuning cache, parses back,
    and computes the transform."""
    import json
    import torch
    from fftgb.plan import Plan
    cache = tmp_path / "tune.json"
    cache.write_text("{}")
    assert lib.fftgb_tune_cache(str(cache).encode()) == 0
    try:
        dims, batch = (4, 512, 512), 1
        p = Plan(dims, batch)
        report = p.autotune(reps=3)
        assert "axis:b8=" in report and "axis=" in report, report
        chosen = report.split("->")[-1].strip()
        assert p.variant == chosen
        assert json.loads(cache.read_text())["512,512,4,1,0"] == chosen
        q = Plan(dims, batch)
        assert q.variant == chosen
        x = orc.uniform_c64(q.points, seed=12)
        y = q(torch.from_numpy(x).to(cuda)).cpu().numpy()
        assert orc.rel_l2(y, orc.c2c_nd(x, dims)) <= TOL
    finally:
        lib.fftgb_tune_cache(b"")

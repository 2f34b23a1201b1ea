"""GPU parity of every entry point against the FP64 oracle.

Tolerance (FP32 path vs FP64 oracle): relative L2 error <= 2e-6, the bound
stated for the plain FP32 form; 1D outputs must also clear the reference's
own pass rule, SNR > 120 dB (examples/helper.cpp:164-198), against the
reference engine's golden vectors.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6


@pytest.fixture(scope="module")
def api(lib, cuda):
    from fftgb import api as a
    return a


@pytest.fixture(scope="module")
def cache_file(tmp_path_factory):
    f = tmp_path_factory.mktemp("plans") / "fftgb_plans.json"
    f.write_text("{}")
    return str(f)


# ------------------------------------------------------------ C ABI, host
@pytest.mark.parametrize("n", [2, 4, 16, 64, 256, 1024, 4096, 8192, 65536])
@pytest.mark.parametrize("inv", [False, True])
def test_c2c_1d(api, n, inv):
    batch = max(1, min(8, (1 << 16) // n))
    x = orc.uniform_c64(n * batch, seed=n + inv)
    y, t = api.c2c_1d(x, n, inv=inv, batch=batch)
    assert t["valid"]
    ref = orc.c2c_1d(x, n, inverse=inv, batch=batch, bit_reversed=True)
    assert orc.rel_l2(y, ref) <= TOL
    assert t["exec_t"] > 0 and t["pcie_write_t"] > 0 and t["pcie_read_t"] > 0


@pytest.mark.parametrize("log_n", range(6, 13))
@pytest.mark.parametrize("inv", [False, True])
def test_c2c_1d_matches_reference_engine(api, log_n, inv):
    g = np.load(os.path.join(ROOT, "tests", "golden", "engine_1d.npz"))
    n = 1 << log_n
    x = g[f"in_{n}"]
    count = int(g[f"count_{n}"])
    y, t = api.c2c_1d(x, n, inv=inv, batch=count)
    assert t["valid"]
    eng = g[f"{'inv' if inv else 'fwd'}_{n}"]
    assert orc.snr_db(y, eng) > 120.0


@pytest.mark.parametrize("inv", [False, True])
def test_host_calls_in_overlapped_chunks(api, lib, inv):
    """Host-buffer calls above 64 MiB run as a chunked copy pipeline (copy-in,
    compute and copy-out of successive chunks overlap), including a short
    last chunk; results equal the oracle, and the fpga_t fields are the
    chunks' summed copy-in, kernel and copy-out times."""
    n, batch = 4096, 2100  # 67 MiB: chunks of 1024, 1024 and 52 transforms
    x = orc.uniform_c64(n * batch, seed=21 + inv)
    y, t = api.c2c_1d(x, n, inv=inv, batch=batch)
    assert t["valid"] and t["exec_t"] > 0
    assert t["pcie_write_t"] > 0 and t["pcie_read_t"] > 0
    assert orc.rel_l2(y, orc.c2c_1d(x, n, inverse=inv, batch=batch, bit_reversed=True)) <= TOL
    n2, how_many = 1024, 9  # 72 MiB: chunks of 4, 4 and 1 grids
    x2 = orc.uniform_c64(n2 * n2 * how_many, seed=22 + inv)
    y2, t2 = api.c2c_2d_bram(x2, n2, inv=inv, how_many=how_many)
    assert t2["valid"] and t2["exec_t"] > 0 and t2["pcie_write_t"] > 0
    assert orc.rel_l2(y2, orc.c2c_nd(x2, (n2, n2), inv, how_many)) <= TOL


@pytest.mark.parametrize("inv", [False, True])
def test_host_3d_grid_in_slabs(api, lib, monkeypatch, inv):
    """One 3D grid above 64 MiB on the per-axis plan runs with its copy-in
    overlapped: x and y passes per slab of planes as the slabs land, then
    the z pass and one contiguous copy-out."""
    monkeypatch.setenv("FFTGB_NO_FUSED", "1")
    lib.fpga_final()  # drop cached plans: the 256^3 plan is rebuilt per axis
    try:
        n = 256
        x = orc.uniform_c64(n ** 3, seed=31 + inv)
        y, t = api.c2c_3d_ddr(x, n, inv=inv)
        assert t["valid"] and t["exec_t"] > 0
        assert t["pcie_write_t"] > 0 and t["pcie_read_t"] > 0
        assert orc.rel_l2(y, orc.c2c_nd(x, (n, n, n), inv)) <= TOL
        # the same grid with input and output in one host buffer
        buf = x.copy()
        t = lib.fftfpgaf_c2c_3d_ddr(n, buf.ctypes.data, buf.ctypes.data, inv)
        assert t.valid
        assert orc.rel_l2(buf, y) <= 1e-7
    finally:
        lib.fpga_final()


def test_host_call_same_and_overlapping_buffers(api, lib):
    """A chunked host call with out == inp transforms in place; buffers that
    overlap partially take the unchunked path (all input read first)."""
    import ctypes
    n, batch = 8192, 1100  # 69 MiB
    x = orc.uniform_c64(n * batch, seed=23)
    ref = orc.c2c_1d(x, n, batch=batch, bit_reversed=True)
    buf = x.copy()
    t = lib.fftfpgaf_c2c_1d(n, buf.ctypes.data, buf.ctypes.data, False, batch)
    assert t.valid
    assert orc.rel_l2(buf, ref) <= TOL
    big = np.zeros(n * batch + 16, dtype=np.complex64)
    big[:n * batch] = x
    t = lib.fftfpgaf_c2c_1d(n, big.ctypes.data, big.ctypes.data + 8 * 16, False, batch)
    assert t.valid
    assert orc.rel_l2(big[16:], ref) <= TOL


def test_c2c_1d_double(api):
    n, batch = 512, 3
    x = orc.uniform_c64(n * batch, seed=3).astype(np.complex128)
    y, t = api.c2c_1d_double(x, n, batch=batch)
    assert t["valid"]
    assert orc.rel_l2(y, orc.c2c_1d(x, n, batch=batch)) <= TOL


@pytest.mark.parametrize("n", [4, 32, 64, 256, 1024])
@pytest.mark.parametrize("inv", [False, True])
def test_c2c_2d(api, n, inv):
    x = orc.uniform_c64(n * n, seed=n)
    y, t = api.c2c_2d_ddr(x, n, inv=inv)
    assert t["valid"]
    assert orc.rel_l2(y, orc.c2c_nd(x, (n, n), inv)) <= TOL
    how_many = 3
    xb = orc.uniform_c64(n * n * how_many, seed=n + 1)
    yb, t = api.c2c_2d_bram(xb, n, inv=inv, how_many=how_many)
    assert t["valid"]
    assert orc.rel_l2(yb, orc.c2c_nd(xb, (n, n), inv, how_many)) <= TOL


@pytest.mark.parametrize("n", [2, 8, 16, 32, 64, 128])
@pytest.mark.parametrize("inv", [False, True])
def test_c2c_3d(api, n, inv):
    x = orc.uniform_c64(n ** 3, seed=n)
    ref = orc.c2c_nd(x, (n, n, n), inv)
    y, t = api.c2c_3d_ddr(x, n, inv=inv)
    assert t["valid"]
    assert orc.rel_l2(y, ref) <= TOL
    y2, t2 = api.c2c_3d_bram(x, n, inv=inv)
    assert t2["valid"]
    assert orc.rel_l2(y2, ref) <= TOL


@pytest.mark.parametrize("n,how_many", [(16, 2), (64, 3), (128, 2)])
def test_c2c_3d_batch(api, n, how_many):
    x = orc.uniform_c64(n ** 3 * how_many, seed=5)
    for inv in (False, True):
        y, t = api.c2c_3d_ddr_batch(x, n, inv=inv, how_many=how_many)
        assert t["valid"] and t["exec_t"] > 0
        assert t["pcie_write_t"] == 0 and t["pcie_read_t"] == 0
        assert orc.rel_l2(y, orc.c2c_nd(x, (n, n, n), inv, how_many)) <= TOL


def test_svm_variants(api, lib, cache_file):
    assert api.initialize("NVIDIA CUDA", cache_file, use_svm=True) == 0
    try:
        n = 32
        x = orc.uniform_c64(n ** 3 * 2, seed=11)
        y, t = api.c2c_3d_ddr_svm(x[: n ** 3], n)
        assert t["valid"]
        assert orc.rel_l2(y, orc.c2c_nd(x[: n ** 3], (n, n, n))) <= TOL
        y, t = api.c2c_3d_ddr_svm_batch(x, n, inv=True, how_many=2)
        assert t["valid"]
        assert orc.rel_l2(y, orc.c2c_nd(x, (n, n, n), True, 2)) <= TOL
        x2 = orc.uniform_c64(64 * 64 * 2, seed=12)
        y, t = api.c2c_2d_bram(x2, 64, how_many=2, svm=True)
        assert t["valid"]
        assert orc.rel_l2(y, orc.c2c_nd(x2, (64, 64), False, 2)) <= TOL
        x1 = orc.uniform_c64(4096 * 2, seed=13)
        y, t = api.c2c_1d(x1, 4096, batch=2, svm=True)
        assert t["valid"]
        assert orc.rel_l2(y, orc.c2c_1d(x1, 4096, batch=2)) <= TOL
    finally:
        api.final()
    # after fpga_final the SVM entry points are invalid again
    y, t = api.c2c_3d_ddr_svm(orc.uniform_c64(8 ** 3, seed=1), 8)
    assert not t["valid"]


def test_c_validity_suite_on_gpu(libpath, cache_file, tmp_path):
    inc = os.path.join(ROOT, "include")
    libdir = os.path.dirname(libpath)
    exe = str(tmp_path / "test_validity")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I" + inc,
                    os.path.join(ROOT, "tests", "c", "test_validity.c"),
                    "-L" + libdir, "-lfftfpga", "-Wl,-rpath," + libdir, "-o", exe],
                   check=True)
    r = subprocess.run([exe, "gpu", cache_file], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def test_input_not_modified(api):
    n = 64
    x = orc.uniform_c64(n ** 3, seed=2)
    x0 = x.copy()
    api.c2c_3d_ddr(x, n)
    assert np.array_equal(x, x0)


# ------------------------------------------------------------ ext API, device
def _torch_c64(x, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


@pytest.mark.parametrize("dims,batch", [
    ((2,), 5), ((64,), 7), ((4096,), 3), ((8192,), 2), ((1 << 16,), 2),
    ((1 << 18,), 1), ((1 << 20,), 1),
    ((8, 4), 3), ((1024, 1024), 1), ((16, 2048), 1), ((512, 64), 2),
    ((4, 8, 16), 2), ((64, 128, 256), 1), ((256, 32, 64), 1), ((32, 32, 32), 4),
])
@pytest.mark.parametrize("inv", [False, True])
def test_plan_natural(cuda, dims, batch, inv):
    from fftgb.plan import Plan
    p = Plan(dims, batch)
    n = int(np.prod(dims)) * batch
    x = orc.uniform_c64(n, seed=len(dims) * 100 + batch)
    y = p(_torch_c64(x, cuda), inverse=inv).cpu().numpy()
    ref = orc.c2c_nd(x, dims, inv, batch)
    assert orc.rel_l2(y, ref) <= TOL


@pytest.mark.parametrize("dims,batch", [
    ((256, 256, 256), 1), ((128, 128, 128), 2), ((64, 64, 64), 3),
    ((32, 32, 32), 2), ((256, 256, 128), 1), ((128, 256, 256), 1),
    ((1024, 1024), 2), ((512, 512), 2), ((128, 128), 5), ((64, 32), 3),
])
@pytest.mark.parametrize("fused", [True, False])
def test_plan_fused_and_generic(cuda, monkeypatch, dims, batch, fused):
    """Two-pass fused plans and per-axis plans give the same transform
    (grids that fit one cluster are kept off the single-launch kernel)."""
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_NO_CLUSTER", "1")
    if not fused:
        monkeypatch.setenv("FFTGB_NO_FUSED", "1")
    p = Plan(dims, batch)
    names = p.pass_names()
    if fused and dims in ((256, 256, 256), (128, 128, 128), (64, 64, 64), (1024, 1024)):
        assert any(nm.startswith("k_xy") for nm in names), names
    if not fused:
        assert not any(nm.startswith(("k_xy", "k_rz")) for nm in names), names
    x = orc.uniform_c64(p.points, seed=sum(dims) + batch)
    xd = _torch_c64(x, cuda)
    for inv in (False, True):
        y = p(xd, inverse=inv).cpu().numpy()
        assert orc.rel_l2(y, orc.c2c_nd(x, dims, inv, batch)) <= TOL, (names, inv)


@pytest.mark.parametrize("dims,batch,nj,x", [
    ((256, 256, 256), 2, 32, 8), ((256, 256, 256), 1, 64, 8), ((256, 256, 256), 1, 32, 4),
    ((256, 256, 256), 1, 64, 16), ((256, 256, 256), 2, 64, 8), ((256, 256, 256), 2, 32, 4),
    ((128, 128, 128), 3, 64, 16), ((128, 128, 128), 2, 128, 32),
    ((64, 64, 64), 5, 64, 32), ((32, 32, 32), 7, 32, 32),
    ((256, 128, 64), 2, 64, 32), ((128, 128, 256), 1, 64, 16),
    ((128, 128, 64), 3, 64, 16),
    ((512, 512), 3, 32, 0), ((256, 256), 4, 64, 0), ((1024, 1024), 2, 16, 0),
])
@pytest.mark.parametrize("pipe", [0, 16, 32, 48])
def test_plan_fused_pipelined(cuda, monkeypatch, dims, batch, nj, x, pipe):
    """The persistent forms of the fused passes (mask 16 / 32: pass A / B
    fed by TMA tensor copies, pass A for rows up to 256 points, pass B for
    (NZ, R, X) = (256, 4, 8), (256, 8, 4) or (128, 2, 16); 0: the one-tile
    kernels) give the transform (rel-L2 vs the FP64 oracle, both directions,
    with and without scaling), including batches with fewer tiles than
    resident CTAs and tiles walked several times per CTA."""
    from fftgb.plan import Plan
    if len(dims) == 2 and pipe == 32:
        pytest.skip("2D plans have no pass B")
    monkeypatch.setenv("FFTGB_FUSED_NJ", str(nj))
    monkeypatch.setenv("FFTGB_FUSED_X", str(x))
    monkeypatch.setenv("FFTGB_FUSED_PIPE", str(pipe))
    p = Plan(dims, batch)
    names = p.pass_names()
    a_name = "k_xy_tma" if pipe & 16 and dims[-1] <= 256 else "k_xy<"
    tma_b = len(dims) == 3 and (dims[0], dims[1] // nj, x) in ((256, 4, 8), (256, 8, 4),
                                                                (128, 2, 16))
    b_name = "k_rz_tma" if pipe & 32 and tma_b else "k_rz<"
    assert names[0].startswith(a_name), names
    if len(dims) == 3:
        assert names[-1].startswith(b_name), names
    xh = orc.uniform_c64(p.points, seed=sum(dims) + nj + x)
    xd = _torch_c64(xh, cuda)
    n = int(np.prod(dims))
    for inv in (False, True):
        y = p(xd, inverse=inv).cpu().numpy()
        assert orc.rel_l2(y, orc.c2c_nd(xh, dims, inv, batch)) <= TOL, (names, inv)
    z = p(p(xd), inverse=True, scale=1.0 / n).cpu().numpy()
    assert orc.rel_l2(z, xh) <= 2 * TOL


@pytest.mark.parametrize("dims,batch", [
    ((128, 256, 64), 2), ((512, 16, 32), 3), ((512, 64), 5), ((256, 128), 3),
    ((256, 256, 256), 1),
])
def test_cols_tma(cuda, monkeypatch, dims, batch):
    """Column passes of 128, 256 and 512 points run in the persistent kernel
    fed by TMA tensor copies (512 points: also written by TMA tensor stores):
    same transform out of place, in place, from an input only 8-byte aligned
    (served by the one-tile kernel) and into an output only 8-byte aligned
    (per-thread stores), both directions, plan status clean."""
    import torch
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_NO_FUSED", "1")
    p = Plan(dims, batch)
    names = p.pass_names()
    assert any(nm.startswith("k_cols_tma") for nm in names), names
    n = p.points
    x = orc.uniform_c64(n, seed=sum(dims) + batch)
    for inv in (False, True):
        ref = orc.c2c_nd(x, dims, inv, batch)
        y = p(_torch_c64(x, cuda), inverse=inv).cpu().numpy()
        assert orc.rel_l2(y, ref) <= TOL, (names, inv)
        if p.pass_names() and len(dims) >= 2:
            buf = _torch_c64(x, cuda)
            p(buf, inverse=inv, out=buf)
            assert orc.rel_l2(buf.cpu().numpy(), ref) <= TOL, ("in place", inv)
        big = torch.zeros(n + 1, dtype=torch.complex64, device=cuda)
        big[1:] = _torch_c64(x, cuda)
        out = torch.zeros(n + 1, dtype=torch.complex64, device=cuda)
        p(big[1:], inverse=inv, out=out[1:])
        assert orc.rel_l2(out[1:].cpu().numpy(), ref) <= TOL, ("unaligned", inv)
        out.zero_()
        p(_torch_c64(x, cuda), inverse=inv, out=out[1:])
        assert orc.rel_l2(out[1:].cpu().numpy(), ref) <= TOL, ("unaligned output", inv)
    assert p.status() == 0


@pytest.mark.parametrize("dims,batch,env,order", [
    ((1 << 16,), 3, {"FFTGB_NO_CLUSTER": "1"}, "bitrev"),    # 256 x 256
    ((1 << 15,), 2, {"FFTGB_NO_CLUSTER": "1"}, "bitrev"),
    ((1 << 17,), 2, {"FFTGB_NO_CLUSTER": "1"}, "bitrev"),
    ((1 << 18,), 1, {"FFTGB_NO_CLUSTER": "1"}, "bitrev"),    # 512 x 512
    ((1 << 16,), 3, {"FFTGB_NO_CLUSTER": "1", "FFTGB_TWIDDLE_PASS1": "1"}, "natural"),
])
def test_cols_tma_twiddled(cuda, monkeypatch, dims, batch, env, order):
    """The TMA-fed column pass with the four-step twiddle on its outputs
    (the first pass of the bit-reversed 1D four-step, which stores in place
    of the columns), against the oracle and against the same plan on the
    one-tile kernel, out of place and from an input only 8-byte aligned."""
    import torch
    from fftgb.plan import Plan
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    p = Plan(dims, batch, order=order)
    names = p.pass_names()
    assert any(nm.startswith("k_cols_tma") for nm in names), names
    monkeypatch.setenv("FFTGB_NO_COLS_TMA", "1")
    q = Plan(dims, batch, order=order)
    assert not any(nm.startswith("k_cols_tma") for nm in q.pass_names())
    n = p.points
    x = orc.uniform_c64(n, seed=sum(dims) + batch + len(order))
    for inv in (False, True):
        if len(dims) == 1:
            ref = orc.c2c_1d(x, dims[0], inv, batch, bit_reversed=order == "bitrev")
        else:
            ref = orc.c2c_nd(x, dims, inv, batch)
        y = p(_torch_c64(x, cuda), inverse=inv).cpu().numpy()
        assert orc.rel_l2(y, ref) <= TOL, (names, inv)
        y1 = q(_torch_c64(x, cuda), inverse=inv).cpu().numpy()
        assert orc.rel_l2(y, y1) <= 1e-6, (names, inv)
        big = torch.zeros(n + 1, dtype=torch.complex64, device=cuda)
        big[1:] = _torch_c64(x, cuda)
        out = torch.zeros(n + 1, dtype=torch.complex64, device=cuda)
        p(big[1:], inverse=inv, out=out[1:])
        assert orc.rel_l2(out[1:].cpu().numpy(), ref) <= TOL, ("unaligned", inv)
    assert p.status() == 0


@pytest.mark.parametrize("pipe", [16, 48])
def test_fused_tma_pass_unaligned_and_in_place(cuda, monkeypatch, pipe):
    """The TMA-fed passes on buffers that are only 8-byte aligned (the
    tensor maps need 16: the one-tile kernels run instead), with only the
    output unaligned, and in a plan executed several times, with the plan's
    status clean."""
    import torch
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_FUSED_NJ", "64")
    monkeypatch.setenv("FFTGB_FUSED_X", "16")
    monkeypatch.setenv("FFTGB_FUSED_PIPE", str(pipe))
    dims, batch = (128, 128, 128), 3
    p = Plan(dims, batch)
    assert p.pass_names()[0].startswith("k_xy_tma"), p.pass_names()
    if pipe & 32:
        assert p.pass_names()[-1].startswith("k_rz_tma"), p.pass_names()
    n = p.points
    x = orc.uniform_c64(n, seed=77)
    big = torch.zeros(n + 1, dtype=torch.complex64, device=cuda)
    big[1:] = _torch_c64(x, cuda)
    out = torch.zeros(n + 1, dtype=torch.complex64, device=cuda)
    for inv in (False, True):
        ref = orc.c2c_nd(x, dims, inv, batch)
        p(big[1:], inverse=inv, out=out[1:])
        assert orc.rel_l2(out[1:].cpu().numpy(), ref) <= TOL
        out.zero_()
        p(_torch_c64(x, cuda), inverse=inv, out=out[1:])  # aligned input only
        assert orc.rel_l2(out[1:].cpu().numpy(), ref) <= TOL
        for _ in range(3):
            y = p(_torch_c64(x, cuda), inverse=inv).cpu().numpy()
        assert orc.rel_l2(y, ref) <= TOL
    assert p.status() == 0


@pytest.mark.parametrize("dims,batch,nj,x", [
    ((256, 256, 256), 1, 32, 8), ((256, 256, 256), 2, 64, 16), ((128, 128, 128), 2, 64, 16),
    ((256, 128, 64), 2, 64, 32), ((64, 64, 64), 3, 64, 32),
    ((1024, 1024), 2, 8, 0), ((512, 512), 3, 16, 0), ((64, 2048), 2, 8, 0),
    ((64, 2048), 3, 4, 0), ((1024, 256), 2, 32, 0),
])
@pytest.mark.parametrize("pipe", [0, 3, 12, 16, 48])
@pytest.mark.parametrize("twiddle_a", [False, True])
def test_fused_y_twiddle_placement(cuda, monkeypatch, dims, batch, nj, x, pipe, twiddle_a):
    """The y twiddle W_ny^(r*k1) of the fused plans multiplied into pass
    B's inputs (default: 3D pass B reads R factors per tile, the 2D column
    pass applies W_ny^(r*(c >> log2 nx)) to its loads) or into pass A's
    outputs (FFTGB_TWIDDLE_A=1), with every form of the passes: same
    transform."""
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_FUSED_NJ", str(nj))
    monkeypatch.setenv("FFTGB_FUSED_X", str(x))
    monkeypatch.setenv("FFTGB_FUSED_PIPE", str(pipe))
    if twiddle_a:
        monkeypatch.setenv("FFTGB_TWIDDLE_A", "1")
    p = Plan(dims, batch)
    assert p.pass_names()[0].startswith("k_xy"), p.pass_names()
    xh = orc.uniform_c64(p.points, seed=sum(dims) + pipe)
    xd = _torch_c64(xh, cuda)
    for inv in (False, True):
        y = p(xd, inverse=inv, scale=0.5).cpu().numpy()
        assert orc.rel_l2(y, 0.5 * orc.c2c_nd(xh, dims, inv, batch)) <= TOL, inv


@pytest.mark.parametrize("dims,batch,nj", [
    ((1024, 1024), 3, 8), ((512, 512), 2, 16), ((64, 2048), 2, 8), ((64, 2048), 3, 4),
    ((8, 1024), 2, 8), ((32, 2048), 1, 4),
])
def test_plan_fused_2d_short_tiles(cuda, monkeypatch, dims, batch, nj):
    """2D pass-A tiles of fewer than 16 rows (the y transform of each column
    in registers, pass B a long column FFT) give the transform."""
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_FUSED_NJ", str(nj))
    p = Plan(dims, batch)
    names = p.pass_names()
    assert names[0] == f"k_xy<{dims[1]},{nj}>", names
    x = orc.uniform_c64(p.points, seed=sum(dims) + nj)
    xd = _torch_c64(x, cuda)
    for inv in (False, True):
        y = p(xd, inverse=inv, scale=0.5 if inv else 1.0).cpu().numpy()
        ref = orc.c2c_nd(x, dims, inv, batch) * (0.5 if inv else 1.0)
        assert orc.rel_l2(y, ref) <= TOL, (names, inv)


def test_plan_2d_defaults(cuda):
    """Measured 2D defaults: axis passes up to 512, 8192-point pass-A tiles
    for wider rows."""
    from fftgb.plan import Plan
    assert Plan((512, 512), 4).variant == "axis"
    assert Plan((1024, 1024), 4).pass_names()[0] == "k_xy<1024,8>"
    assert Plan((2048, 2048), 1).pass_names()[0] == "k_xy<2048,4>"
    # rows of 1024 over 512-point columns: axis passes on a large batch
    # (the column pass is the TMA kernel), the fused tile for one grid
    assert Plan((512, 1024), 128).variant == "axis"
    assert Plan((512, 1024), 1).variant.startswith("fused")


@pytest.mark.parametrize("n,batch", [(1 << 13, 9), (1 << 14, 2), (1 << 15, 3), (1 << 16, 4),
                                     (1 << 17, 3), (1 << 18, 2), (1 << 19, 1), (1 << 20, 1),
                                     (1 << 21, 1)])
@pytest.mark.parametrize("form", ["rows", "cols", "cols_tw1"])
def test_four_step_forms(cuda, monkeypatch, n, batch, form):
    """The natural-order four-step in its forms, both directions, scaled:
    "rows" (default where rows of L1 <= 1024 points exist): the column pass
    keeps its layout and twiddles its outputs, then a row pass stores the
    transposed order through shared memory; "cols" (FFTGB_1D_COLS=1): a
    transposed column store, then a column pass with the twiddle on its
    loads (FFTGB_TWIDDLE_PASS1=1: on the first pass's stores instead)."""
    import torch
    from fftgb import _lib
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_NO_CLUSTER", "1")
    if form != "rows":
        monkeypatch.setenv("FFTGB_1D_COLS", "1")
    if form == "cols_tw1":
        monkeypatch.setenv("FFTGB_TWIDDLE_PASS1", "1")
    p = Plan((n,), batch)
    names = p.pass_names()
    lg = n.bit_length() - 1
    l1, l2 = 1 << (lg - lg // 2), 1 << (lg // 2)
    if form == "rows" and l1 <= 1024:
        assert names[0] in (f"k_cols_tma<{l2}>", f"k_cols<{l2}>") and \
            names[1] == f"k_rows<{l1}>", names
    else:
        assert names[0] == f"k_cols<{l2}>" and \
            names[1] in (f"k_cols<{l1}>", f"k_cols_tma<{l1}>"), names
    x = orc.uniform_c64(n * batch, seed=n + batch)
    xd = _torch_c64(x, cuda)
    for inv in (False, True):
        y = p(xd, inverse=inv, scale=0.25).cpu().numpy()
        ref = 0.25 * orc.c2c_1d(x, n, inverse=inv, batch=batch, bit_reversed=False)
        assert orc.rel_l2(y, ref) <= TOL, (names, inv)
    if form == "rows" and n in (1 << 16, 1 << 18):
        # buffers only 8-byte aligned (the column pass falls back to the
        # one-tile kernel), and in place refused (the row pass scatters)
        big = torch.zeros(n * batch + 1, dtype=torch.complex64, device=cuda)
        big[1:] = xd
        out = torch.zeros_like(big)
        p(big[1:], out=out[1:])
        ref = orc.c2c_1d(x, n, batch=batch, bit_reversed=False)
        assert orc.rel_l2(out[1:].cpu().numpy(), ref) <= TOL
        with pytest.raises(_lib.FFTGBError):
            p(xd, out=xd)


@pytest.mark.parametrize("n", [1 << 15, 1 << 16, 1 << 17])
@pytest.mark.parametrize("order", ["natural", "bitrev"])
@pytest.mark.parametrize("cluster", [True, False])
def test_1d_cluster_and_four_step(cuda, monkeypatch, n, order, cluster):
    """Single-pass cluster kernel and two-pass four-step give the same 1D
    transform in both output orders."""
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_CLUSTER" if cluster else "FFTGB_NO_CLUSTER", "1")
    batch = 3
    p = Plan((n,), batch, order=order)
    names = p.pass_names()
    assert any(nm.startswith(("k_1d_cluster", "k_1d_push")) for nm in names) == cluster, names
    x = orc.uniform_c64(n * batch, seed=n + cluster)
    xd = _torch_c64(x, cuda)
    for inv in (False, True):
        y = p(xd, inverse=inv, scale=0.5).cpu().numpy()
        ref = 0.5 * orc.c2c_1d(x, n, inverse=inv, batch=batch,
                               bit_reversed=(order == "bitrev"))
        assert orc.rel_l2(y, ref) <= TOL, (names, inv)


@pytest.mark.parametrize("n,csize", [(1 << 15, 2), (1 << 15, 8), (1 << 16, 4), (1 << 16, 8),
                                     (1 << 16, 16), (1 << 17, 8), (1 << 17, 16)])
@pytest.mark.parametrize("order", ["natural", "bitrev"])
@pytest.mark.parametrize("form", [0, 1])
def test_1d_cluster_sizes(cuda, monkeypatch, n, csize, order, form):
    """Every instantiated cluster size gives the transform (16-CTA clusters
    use the non-portable cluster size), with each exchange form that exists
    for it: remote loads (0), bulk copies (1)."""
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_CLUSTER", "1")
    monkeypatch.setenv("FFTGB_CLUSTER_SIZE", str(csize))
    monkeypatch.setenv("FFTGB_C1D_FORM", str(form))
    batch = 5
    p = Plan((n,), batch, order=order)
    names = p.pass_names()
    bulk = (n, csize) in ((1 << 16, 16), (1 << 15, 8))
    kern = ["k_1d_cluster", "k_1d_push"][form] if bulk else "k_1d_cluster"
    l1 = 256 if n < (1 << 17) else 512
    assert names == [f"{kern}<{l1},{n // l1},{csize}>"], names
    assert p.variant == f"cluster:{csize}"
    x = orc.uniform_c64(n * batch, seed=n + csize)
    xd = _torch_c64(x, cuda)
    for inv in (False, True):
        y = p(xd, inverse=inv).cpu().numpy()
        ref = orc.c2c_1d(x, n, inverse=inv, batch=batch, bit_reversed=(order == "bitrev"))
        assert orc.rel_l2(y, ref) <= TOL, (names, inv)
    assert p.status() == 0


@pytest.mark.parametrize("n,csize,batch", [(1 << 16, 16, 67), (1 << 15, 8, 203)])
@pytest.mark.parametrize("order", ["natural", "bitrev"])
def test_1d_push_large_batch(cuda, monkeypatch, n, csize, batch, order):
    """The bulk-copy cluster kernel over more clusters than are resident at
    once, out of place, in place, and on an input and output that are only
    8-byte aligned (the copies move shared memory only)."""
    import torch
    from fftgb.plan import Plan
    monkeypatch.setenv("FFTGB_CLUSTER", "1")
    monkeypatch.setenv("FFTGB_CLUSTER_SIZE", str(csize))
    monkeypatch.setenv("FFTGB_C1D_FORM", "1")
    p = Plan((n,), batch, order=order)
    assert p.pass_names()[0].startswith("k_1d_push"), p.pass_names()
    x = orc.uniform_c64(n * batch, seed=batch)
    br = order == "bitrev"
    for inv in (False, True):
        ref = orc.c2c_1d(x, n, inverse=inv, batch=batch, bit_reversed=br)
        y = p(_torch_c64(x, cuda), inverse=inv).cpu().numpy()
        assert orc.rel_l2(y, ref) <= TOL, ("out of place", inv)
        buf = _torch_c64(x, cuda)
        p(buf, inverse=inv, out=buf)
        assert orc.rel_l2(buf.cpu().numpy(), ref) <= TOL, ("in place", inv)
        big = torch.zeros(n * batch + 1, dtype=torch.complex64, device=cuda)
        big[1:] = _torch_c64(x, cuda)
        out = torch.zeros(n * batch + 1, dtype=torch.complex64, device=cuda)
        p(big[1:], inverse=inv, out=out[1:])
        assert orc.rel_l2(out[1:].cpu().numpy(), ref) <= TOL, ("unaligned", inv)
        assert p.status() == 0


@pytest.mark.parametrize("dims,batch,env,order", [
    # four-step pass 2 (a plain column pass when the twiddle stays in pass 1)
    ((1 << 16,), 5, {"FFTGB_NO_CLUSTER": "1", "FFTGB_TWIDDLE_PASS1": "1"}, "natural"),
    ((1 << 16,), 3, {"FFTGB_NO_CLUSTER": "1"}, "bitrev"),    # pass 1 with twiddle
    ((1 << 17,), 2, {"FFTGB_NO_CLUSTER": "1", "FFTGB_TWIDDLE_PASS1": "1"}, "natural"),
    ((1 << 13,), 7, {"FFTGB_NO_CLUSTER": "1", "FFTGB_TWIDDLE_PASS1": "1"}, "natural"),
    # fused 2D pass B with the y twiddle left in pass A
    ((1024, 1024), 3, {"FFTGB_TWIDDLE_A": "1"}, "natural"),
    ((256, 512), 2, {"FFTGB_NO_FUSED": "1"}, "natural"),      # 2D axis passes
    ((64, 128, 256), 2, {"FFTGB_NO_FUSED": "1"}, "natural"),  # y and z passes
    ((256, 64, 512), 1, {"FFTGB_NO_FUSED": "1"}, "natural"),
    ((128, 512, 64), 1, {"FFTGB_NO_FUSED": "1"}, "natural"),
])
def test_cols_variants(cuda, monkeypatch, dims, batch, env, order):
    """Column passes in their plan variants (four-step with the twiddle on
    either pass, fused 2D pass B, per-axis passes; k_cols or the TMA-fed
    k_cols_tma) give the transform (both directions, scaled inverse)."""
    from fftgb.plan import Plan
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    p = Plan(dims, batch, order=order)
    names = p.pass_names()
    assert any(nm.startswith("k_cols") for nm in names), names
    x = orc.uniform_c64(p.points, seed=sum(dims) + batch + len(order))
    xd = _torch_c64(x, cuda)
    n = int(np.prod(dims))
    for inv in (False, True):
        y = p(xd, inverse=inv, scale=1.0 / n if inv else 1.0).cpu().numpy()
        if len(dims) == 1:
            ref = orc.c2c_1d(x, n, inverse=inv, batch=batch, bit_reversed=(order == "bitrev"))
        else:
            ref = orc.c2c_nd(x, dims, inv, batch)
        if inv:
            ref = ref / n
        assert orc.rel_l2(y, ref) <= TOL, (names, inv)


@pytest.mark.parametrize("n", [8, 1024, 8192, 1 << 16])
def test_plan_bitrev_and_adjoint(cuda, n):
    import torch
    from fftgb.plan import Plan
    batch = 2
    p = Plan((n,), batch, order="bitrev")
    x = orc.uniform_c64(n * batch, seed=n)
    xd = _torch_c64(x, cuda)
    y = p(xd).cpu().numpy()
    assert orc.rel_l2(y, orc.c2c_1d(x, n, batch=batch, bit_reversed=True)) <= TOL
    # adjoint: <A x, z> == <x, A^H z>
    z = orc.uniform_c64(n * batch, seed=n + 1)
    zd = _torch_c64(z, cuda)
    ahz = p.execute(zd, adjoint=True).cpu().numpy().astype(np.complex128)
    lhs = np.vdot(z.astype(np.complex128), y.astype(np.complex128))
    rhs = np.vdot(ahz, x.astype(np.complex128))
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)
    # adjoint of the forward = unnormalised inverse of the un-bit-reversed input
    perm = orc.bitrev_perm(n.bit_length() - 1)
    zr = z.reshape(batch, n)[:, perm].reshape(-1)
    ref = orc.c2c_nd(zr, (n,), True, batch)
    assert orc.rel_l2(ahz, ref) <= TOL
    torch.cuda.synchronize()


def test_plan_scale_and_adjoint_natural(cuda):
    from fftgb.plan import Plan
    dims = (16, 32, 8)
    p = Plan(dims, 2)
    x = orc.uniform_c64(p.points, seed=9)
    xd = _torch_c64(x, cuda)
    y = p(xd, scale=0.25).cpu().numpy()
    assert orc.rel_l2(y, 0.25 * orc.c2c_nd(x, dims, False, 2)) <= TOL
    ya = p.execute(xd, adjoint=True).cpu().numpy()
    assert orc.rel_l2(ya, orc.c2c_nd(x, dims, True, 2)) <= TOL
    yai = p.execute(xd, inverse=True, adjoint=True).cpu().numpy()
    assert orc.rel_l2(yai, orc.c2c_nd(x, dims, False, 2)) <= TOL


def test_plan_inplace(cuda):
    from fftgb.plan import Plan
    p = Plan((64, 64), 2)
    x = orc.uniform_c64(p.points, seed=4)
    xd = _torch_c64(x, cuda)
    p(xd, out=xd)
    assert orc.rel_l2(xd.cpu().numpy(), orc.c2c_nd(x, (64, 64), False, 2)) <= TOL


# ------------------------------------------------------------ full sizes
def test_256cubed_batch8_properties(cuda):
    """256^3 x 8 (the headline workload): one grid against the oracle, all
    grids through size-independent properties (round trip, Parseval,
    linearity)."""
    import torch
    from fftgb.plan import Plan
    n, b = 256, 8
    p = Plan((n, n, n), b)
    g = torch.Generator(device=cuda).manual_seed(2)
    x = (torch.rand(p.points, 2, device=cuda, generator=g) * 2 - 1)
    x = torch.view_as_complex(x.contiguous())
    y = p(x)
    # grid 3 against the FP64 oracle
    g3 = slice(3 * n ** 3, 4 * n ** 3)
    ref = orc.c2c_nd(x[g3].cpu().numpy(), (n, n, n))
    assert orc.rel_l2(y[g3].cpu().numpy(), ref) <= TOL
    # Parseval per grid: sum|Y|^2 = N^3 sum|X|^2
    ex = (x.abs() ** 2).double().view(b, -1).sum(1)
    ey = (y.abs() ** 2).double().view(b, -1).sum(1)
    assert torch.allclose(ey, ex * n ** 3, rtol=1e-5)
    # round trip
    z = p(y, inverse=True, scale=1.0 / n ** 3)
    err = ((z - x).abs() ** 2).double().sum().sqrt() / (x.abs() ** 2).double().sum().sqrt()
    assert err.item() <= TOL
    # linearity: F(x + 2 y) = F(x) + 2 F(y)
    y2 = p(x + 2 * z)
    lin = ((y2 - y - 2 * p(z)).abs() ** 2).double().sum().sqrt() / (y2.abs() ** 2).double().sum().sqrt()
    assert lin.item() <= 4 * TOL


def test_512cubed_round_trip(cuda):
    import torch
    from fftgb.plan import Plan
    n = 512
    p = Plan((n, n, n), 1)
    g = torch.Generator(device=cuda).manual_seed(3)
    x = torch.view_as_complex((torch.rand(p.points, 2, device=cuda, generator=g) * 2 - 1).contiguous())
    y = p(x)
    # one z-pencil-heavy spot check against the oracle: plane sums are the
    # kz = 0 slice of the 2D transform of the z-summed grid
    xs = x.view(n, n, n).sum(0).cpu().numpy().astype(np.complex128)
    ref = np.fft.fft2(xs)
    assert orc.rel_l2(y.view(n, n, n)[0].cpu().numpy(), ref) <= 4 * TOL
    z = p(y, inverse=True, scale=1.0 / n ** 3)
    err = ((z - x).abs() ** 2).double().sum().sqrt() / (x.abs() ** 2).double().sum().sqrt()
    assert err.item() <= TOL
    del x, y, z
    torch.cuda.empty_cache()


def test_autotune_and_cache(cuda, lib, tmp_path):
    """The autotuner times every decomposition, keeps the fastest, and the
    JSON cache makes later plans of the shape start with that choice."""
    import json
    from fftgb.plan import Plan
    cache = tmp_path / "tune.json"
    cache.write_text("{}")
    assert lib.fftgb_tune_cache(str(cache).encode()) == 0
    try:
        dims, batch = (64, 64, 64), 4
        p = Plan(dims, batch)
        report = p.autotune(reps=3)
        assert "->" in report and "axis=" in report, report
        chosen = report.split("->")[-1].strip()
        assert p.variant == chosen
        x = orc.uniform_c64(p.points, seed=21)
        y = p(_torch_c64(x, cuda)).cpu().numpy()
        assert orc.rel_l2(y, orc.c2c_nd(x, dims, False, batch)) <= TOL
        saved = json.loads(cache.read_text())
        assert saved["64,64,64,4,0"] == chosen
        assert Plan(dims, batch).variant == chosen
        p1 = Plan((1 << 16,), 8)
        r1 = p1.autotune(reps=3)
        assert "fourstep=" in r1 and "cluster:4=" in r1, r1
        assert p1.variant == r1.split("->")[-1].strip()
        x1 = orc.uniform_c64(p1.points, seed=22)
        y1 = p1(_torch_c64(x1, cuda)).cpu().numpy()
        assert orc.rel_l2(y1, orc.c2c_nd(x1, (1 << 16,), False, 8)) <= TOL
    finally:
        lib.fftgb_tune_cache(b"")

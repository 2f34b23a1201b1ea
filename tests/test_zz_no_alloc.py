"""fftgb_c2c_1d_noalloc: the allocation-free 1D entry point.

Some callers cannot call cudaMalloc: applications whose device memory is
owned by their own pool allocator, and hot paths that must not allocate
because cudaMalloc can synchronise the device.  fftgb_c2c_1d_noalloc serves
them with a file-scope device scratch array instead of allocations.  This
test calls it through the C ABI twice in a row and checks each result
against the regular entry point (a bit-reversed fftgb_plan_1d executed with
fftgb_exec), within the parity tolerance used by the other GPU tests.

The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _regular(lib, torch, x, n, batch, inverse):
    h = ctypes.c_void_p()
    assert lib.fftgb_plan_1d(ctypes.byref(h), n, batch, 0x1) == 0
    try:
        y = torch.empty_like(x)
        assert lib.fftgb_exec(h, x.data_ptr(), y.data_ptr(), inverse, 1.0, None) == 0
        torch.cuda.synchronize()
        return y.cpu().numpy()
    finally:
        lib.fftgb_plan_destroy(h)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n,batch,inverse", [
    (1 << 16, 40, 0),   # 2.6 M points: three rounds through the 1 M-point scratch
    (1 << 20, 2, 1),    # the largest supported n, two rounds
    (8192, 5, 0),
    (1024, 7, 1),       # single pass, no scratch
])
def test_noalloc_matches_regular_entry_point(lib, cuda, n, batch, inverse):
    import torch
    outs = []
    for call in range(2):  # two calls in a row share the scratch
        x = torch.from_numpy(orc.uniform_c64(n * batch, seed=100 * call + n % 97)).to(cuda)
        y = torch.empty_like(x)
        rc = lib.fftgb_c2c_1d_noalloc(n, batch, x.data_ptr(), y.data_ptr(), inverse, None)
        assert rc == 0, lib.fftgb_noalloc_last_error().decode()
        torch.cuda.synchronize()
        got = y.cpu().numpy()
        want = _regular(lib, torch, x, n, batch, inverse)
        assert _rel(got, want) <= TOL
        outs.append(got)
    assert not np.array_equal(outs[0], outs[1])


def test_noalloc_against_oracle(lib, cuda):
    import torch
    n, batch = 1 << 14, 3
    xh = orc.uniform_c64(n * batch, seed=5)
    x = torch.from_numpy(xh).to(cuda)
    y = torch.empty_like(x)
    assert lib.fftgb_c2c_1d_noalloc(n, batch, x.data_ptr(), y.data_ptr(), 0, None) == 0
    torch.cuda.synchronize()
    assert orc.rel_l2(y.cpu().numpy(), orc.c2c_1d(xh, n, batch=batch)) <= TOL


def test_noalloc_rejects_bad_sizes(lib, cuda):
    import torch
    x = torch.zeros(16, dtype=torch.complex64, device=cuda)
    y = torch.zeros_like(x)
    assert lib.fftgb_c2c_1d_noalloc(1 << 21, 1, x.data_ptr(), y.data_ptr(), 0, None) == -5
    assert b"2^20" in lib.fftgb_noalloc_last_error()
    assert lib.fftgb_c2c_1d_noalloc(12, 1, x.data_ptr(), y.data_ptr(), 0, None) == -1
    assert lib.fftgb_c2c_1d_noalloc(16, 1, x.data_ptr(), x.data_ptr(), 0, None) == -1
    assert lib.fftgb_c2c_1d_noalloc(16, 0, x.data_ptr(), y.data_ptr(), 0, None) == -1

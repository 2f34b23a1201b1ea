"""Timeout reporting of the bounded device-side waits.

Every kernel that waits on the device (TMA tile copies, the cluster 1D
kernel's bulk-copy exchange, tensor-core MMA completion, the ragged work
list's dependency counters) gives up after a bounded number of polls,
records the timeout in its family's status word and returns.  A test must
not make a real copy's wait run out: the kernel would then go on while the
copy is still in flight.  So each family's give-up path is run on its own
through fftgb_debug_expire_wait / fftgb_ragged_debug_expire: one thread
waits on an mbarrier (a counter) that nothing ever completes, gives up after
a few polls and sets the same status word.  The tests then check that

* fftgb_plan_status / fftgb_ragged_status of a plan using that family
  reports FFTGB_ETIMEOUT once and then FFTGB_OK (the flag is cleared);
* the reference-facing calls return valid = false after such a timeout and
  valid = true, with correct results, on the next call;
* the plan still computes correct results afterwards (rel-L2 <= 2e-6
  against the FP64 oracle).
"""
import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu

TOL = 2e-6
POLLS = 1000


def _family_plans():
    from fftgb import _lib
    # (wait family, plan dims slowest first, batch, precision, kernel name)
    return [
        (_lib.WAIT_COLS_TMA, (128, 512, 512), 1, "fp32", "k_cols_tma"),
        (_lib.WAIT_FUSED_TMA, (256, 256, 256), 1, "fp32", "k_rz_tma"),
        (_lib.WAIT_CLUSTER_1D, (65536,), 8, "fp32", "k_1d_push"),
        (_lib.WAIT_TENSOR_CORE, (16, 256, 256), 1, "tc_fp16", "_tc"),
    ]


@pytest.mark.parametrize("case", range(4))
def test_plan_status_reports_and_clears(cuda, case):
    import torch
    from fftgb import _lib
    from fftgb.plan import Plan
    fam, dims, batch, prec, kname = _family_plans()[case]
    p = Plan(dims, batch, precision=prec)
    names = p.pass_names()
    assert any(kname in n for n in names), names
    x = orc.uniform_c64(p.points, seed=21 + case)
    xd = torch.from_numpy(x).to(cuda)
    p(xd)
    assert p.status() == _lib.OK
    L = _lib.lib()
    assert L.fftgb_debug_expire_wait(fam, POLLS) == _lib.OK
    assert p.status() == _lib.ETIMEOUT, names
    assert "gave up" in _lib.last_error()
    assert p.status() == _lib.OK  # cleared by the first read
    y = p(xd).cpu().numpy()
    assert p.status() == _lib.OK
    ref = orc.c2c_nd(x, dims, False, batch) if len(dims) > 1 else \
        orc.c2c_1d(x, dims[0], batch=batch, bit_reversed=False)
    assert orc.rel_l2(y, ref) <= TOL


def test_unknown_family_rejected(cuda):
    from fftgb import _lib
    L = _lib.lib()
    assert L.fftgb_debug_expire_wait(99, POLLS) == _lib.EINVAL
    assert L.fftgb_debug_expire_wait(_lib.WAIT_COLS_TMA, (1 << 20) + 1) == _lib.EINVAL


def test_abi_call_invalid_after_timeout(cuda):
    """fftfpgaf_c2c_3d_ddr on a 256^3 grid runs the TMA-fed pass B: a
    timeout of that family turns the next call's result into valid = false;
    the call after it is valid again and correct."""
    from fftgb import _lib, api
    from fftgb.plan import Plan
    n = 256
    assert any("k_rz_tma" in s for s in Plan((n, n, n), 1).pass_names())
    x = orc.uniform_c64(n ** 3, seed=31)
    _, t = api.c2c_3d_ddr(x, n)
    assert t["valid"]
    assert _lib.lib().fftgb_debug_expire_wait(_lib.WAIT_FUSED_TMA, POLLS) == _lib.OK
    _, t = api.c2c_3d_ddr(x, n)
    assert not t["valid"]
    y, t = api.c2c_3d_ddr(x, n)
    assert t["valid"]
    assert orc.rel_l2(y, orc.c2c_nd(x, (n, n, n))) <= TOL


def test_ragged_status_reports_and_clears(cuda):
    import torch
    from fftgb import _lib
    from fftgb.plan import RaggedPlan
    shapes = [(32, 64, 128), (64, 64, 64), (16, 32, 16)]
    rp = RaggedPlan(shapes)
    assert rp.launches == 1
    x = orc.uniform_c64(rp.points, seed=41)
    xd = torch.from_numpy(x).to(cuda)
    rp(xd)
    assert rp.status() == _lib.OK
    assert _lib.lib().fftgb_ragged_debug_expire(rp._h, POLLS) == _lib.OK
    assert rp.status() == _lib.ETIMEOUT
    assert rp.status() == _lib.OK
    y = rp(xd).cpu().numpy()
    assert rp.status() == _lib.OK
    off = 0
    for s in shapes:
        m = int(np.prod(s))
        assert orc.rel_l2(y[off:off + m], orc.c2c_nd(x[off:off + m], s)) <= TOL
        off += m


def test_ragged_grouped_status_reports_and_clears(cuda):
    """A ragged plan whose 256 x 256 x 128 grids run as grouped TMA-fed
    passes reports a give-up of that wait family through
    fftgb_ragged_status, once, and stays correct."""
    import torch
    from fftgb import _lib
    from fftgb.plan import RaggedPlan
    shapes = [(64, 64, 64), (256, 256, 128), (32, 32, 32)]
    rp = RaggedPlan(shapes)
    assert rp.launches == 3
    x = orc.uniform_c64(rp.points, seed=43)
    xd = torch.from_numpy(x).to(cuda)
    rp(xd)
    assert rp.status() == _lib.OK
    assert _lib.lib().fftgb_debug_expire_wait(_lib.WAIT_FUSED_TMA, POLLS) == _lib.OK
    assert rp.status() == _lib.ETIMEOUT
    assert rp.status() == _lib.OK
    y = rp(xd).cpu().numpy()
    assert rp.status() == _lib.OK
    off = 0
    for s in shapes:
        m = int(np.prod(s))
        assert orc.rel_l2(y[off:off + m], orc.c2c_nd(x[off:off + m], s)) <= TOL
        off += m

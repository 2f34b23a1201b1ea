"""Differentiation: the adjoint kernels behind torch.autograd.

Workload: a spectral Poisson-filter loss, phi = IFFT3(FFT3(rho) G) / N^3 with
G = 1/|k|^2 (G(0) = 0), loss = sum |phi - phi_t|^2, on seeded Gaussian
fields whose spectrum decays as |k|^-3.

* gradcheck against FP64 finite differences at 16^3 (the loss is quadratic,
  so central differences carry no truncation error; tolerances cover the
  FP32 kernels' rounding);
* the autograd gradient at 4 x 128^3 against the analytic gradient
  2 A^H (A rho - phi_t), A = F^H diag(G) F / N^3, evaluated in FP64 numpy.
"""
import numpy as np
import pytest

from oracle import fft_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ag(lib, cuda):
    from fftgb import autograd
    return autograd


def _fields(dims, batch, seed):
    from fftgb import synthetic
    return synthetic.spectral_field(dims, batch, seed=seed).reshape((batch,) + dims)


def test_fftn_backward_is_adjoint(ag, cuda):
    import torch
    dims = (8, 16, 32)
    x = torch.from_numpy(orc.uniform_c64(2 * 8 * 16 * 32, seed=1).reshape((2,) + dims)).to(cuda)
    x.requires_grad_(True)
    y = ag.fftn(x, dims)
    w = torch.from_numpy(orc.uniform_c64(y.numel(), seed=2).reshape(y.shape)).to(cuda)
    # L = Re <w, y>  ->  grad_x = A^H w (PyTorch's conjugate-Wirtinger convention)
    (torch.real(torch.sum(torch.conj(w) * y))).backward()
    ref = orc.c2c_nd(w.cpu().numpy(), dims, inverse=True, batch=2)
    assert orc.rel_l2(x.grad.cpu().numpy(), ref) <= 2e-6


def test_gradcheck_poisson_16(ag, cuda):
    import torch
    dims = (16, 16, 16)
    g = ag.poisson_filter(dims).to(cuda)
    rho = torch.from_numpy(_fields(dims, 1, 9).astype(np.complex128)).to(cuda)
    phit = torch.from_numpy(_fields(dims, 1, 10).astype(np.complex128)).to(cuda)
    rho.requires_grad_(True)
    f = lambda r: ag.poisson_loss(r, phit, g)
    assert torch.autograd.gradcheck(f, (rho,), eps=5e-2, atol=2e-3, rtol=2e-3,
                                    fast_mode=True)


def test_poisson_gradient_4x128(ag, cuda):
    import torch
    dims = (128, 128, 128)
    n = 128 ** 3
    g = ag.poisson_filter(dims)
    rho_np = _fields(dims, 4, 9)
    phit_np = _fields(dims, 4, 10)
    rho = torch.from_numpy(rho_np).to(cuda).requires_grad_(True)
    phit = torch.from_numpy(phit_np).to(cuda)
    loss = ag.poisson_loss(rho, phit, g.to(cuda))
    loss.backward()
    # analytic FP64 gradient
    G = g.numpy().astype(np.float64)
    r = rho_np.astype(np.complex128)
    phi = np.fft.ifftn(np.fft.fftn(r, axes=(1, 2, 3)) * G, axes=(1, 2, 3))
    res = phi - phit_np
    grad = 2.0 * np.fft.ifftn(np.fft.fftn(res, axes=(1, 2, 3)) * G, axes=(1, 2, 3))
    loss_ref = float(np.sum(np.abs(res) ** 2))
    assert abs(loss.item() - loss_ref) <= 1e-5 * loss_ref
    assert orc.rel_l2(rho.grad.cpu().numpy(), grad) <= 1e-5
    del n


# ---------------------------------------------------------- fused filter
def _g64(dims):
    ks = np.meshgrid(*[np.fft.fftfreq(d, d=1.0 / d) for d in dims], indexing="ij")
    k2 = sum(k ** 2 for k in ks)
    return np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)


@pytest.mark.parametrize("dims,batch,env", [
    ((128, 128, 128), 4, {}),                       # fused plan, TMA pass B
    ((64, 64, 64), 2, {}),                          # fused plan, one-tile pass B
    ((32, 32, 32), 3, {}),                          # single-launch cluster plan
    ((64, 128, 256), 1, {"FFTGB_NO_FUSED": "1"}),   # per-axis plan
    ((16, 32, 64), 2, {"FFTGB_NO_CLUSTER": "1"}),
])
def test_exec_filtered(cuda, monkeypatch, dims, batch, env):
    """filter(transform(x)) and filter(adjoint(x)) against G . FFT in FP64,
    whichever pass (or the extra element-wise kernel) applies G."""
    import torch
    from fftgb.plan import Plan
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    p = Plan(dims, batch)
    x = orc.uniform_c64(p.points, seed=sum(dims))
    xd = torch.from_numpy(x).to(cuda)
    G = np.tile(_g64(dims).reshape(-1), batch)
    for inv in (False, True):
        y = p.execute(xd, inverse=inv, filter="poisson").cpu().numpy()
        ref = G * orc.c2c_nd(x, dims, inv, batch)
        assert orc.rel_l2(y, ref) <= 2e-6, (dims, inv, p.pass_names())
    ya = p.execute(xd, inverse=False, adjoint=True, scale=0.5, filter="poisson").cpu().numpy()
    assert orc.rel_l2(ya, 0.5 * G * orc.c2c_nd(x, dims, True, batch)) <= 2e-6


@pytest.mark.parametrize("dims,batch", [((128, 128, 128), 4), ((96, 100, 90), 2)])
def test_fused_poisson_matches_fp64_and_unfused(ag, cuda, dims, batch):
    """The fused loss (filter inside the transforms, residual and sum of
    squares in one kernel, backward through the adjoint kernels) against the
    analytic FP64 loss and gradient at 4 x 128^3 and on a grid of sides
    2^a 3^b 5^c (mixed-radix plans, the filter as its own pass), and against
    the unfused autograd path."""
    import torch
    g = ag.poisson_filter(dims)
    rho_np = _fields(dims, batch, 9)
    phit_np = _fields(dims, batch, 10)
    rho = torch.from_numpy(rho_np).to(cuda).requires_grad_(True)
    phit = torch.from_numpy(phit_np).to(cuda).requires_grad_(True)
    loss = ag.poisson_loss_fused(rho, phit)
    loss.backward()
    G = g.numpy().astype(np.float64)
    r = rho_np.astype(np.complex128)
    res = np.fft.ifftn(np.fft.fftn(r, axes=(1, 2, 3)) * G, axes=(1, 2, 3)) - phit_np
    grad = 2.0 * np.fft.ifftn(np.fft.fftn(res, axes=(1, 2, 3)) * G, axes=(1, 2, 3))
    loss_ref = float(np.sum(np.abs(res) ** 2))
    assert loss.dtype == torch.float32 and loss.dim() == 0
    assert abs(loss.item() - loss_ref) <= 1e-5 * loss_ref
    assert orc.rel_l2(rho.grad.cpu().numpy(), grad) <= 1e-5
    assert orc.rel_l2(phit.grad.cpu().numpy(), -2.0 * res) <= 1e-5
    # same as the unfused path, and a second backward with a scaled output
    rho2 = torch.from_numpy(rho_np).to(cuda).requires_grad_(True)
    l2 = ag.poisson_loss(rho2, phit.detach(), g.to(cuda))
    l2.backward()
    assert abs(l2.item() - loss.item()) <= 1e-5 * loss_ref
    assert orc.rel_l2(rho2.grad.cpu().numpy(), rho.grad.cpu().numpy()) <= 1e-5
    rho.grad = None
    (3.0 * ag.poisson_loss_fused(rho, phit.detach())).backward()
    assert orc.rel_l2(rho.grad.cpu().numpy(), 3.0 * grad) <= 1e-5


def test_gradcheck_poisson_fused_16(ag, cuda):
    import torch
    dims = (16, 16, 16)
    rho = torch.from_numpy(_fields(dims, 1, 9).astype(np.complex128)).to(cuda)
    phit = torch.from_numpy(_fields(dims, 1, 10).astype(np.complex128)).to(cuda)
    rho.requires_grad_(True)
    f = lambda r: ag.poisson_loss_fused(r, phit)
    assert torch.autograd.gradcheck(f, (rho,), eps=5e-2, atol=2e-3, rtol=2e-3,
                                    fast_mode=True)


def test_residual_sq(lib, cuda):
    import ctypes
    import torch
    n = 1_000_003
    a = torch.from_numpy(orc.uniform_c64(n, seed=1)).to(cuda)
    b = torch.from_numpy(orc.uniform_c64(n, seed=2)).to(cuda)
    r = torch.empty_like(a)
    acc = torch.zeros(1, dtype=torch.float64, device=cuda)
    s = torch.cuda.current_stream()
    assert lib.fftgb_residual_sq(a.data_ptr(), b.data_ptr(), r.data_ptr(), n,
                                 acc.data_ptr(), s.cuda_stream) == 0
    d = (a - b).cpu().numpy().astype(np.complex128)
    assert orc.rel_l2(r.cpu().numpy(), d) <= 1e-7
    assert abs(acc.item() - float(np.sum(np.abs(d) ** 2))) <= 1e-6 * acc.item()
    assert lib.fftgb_residual_sq(a.data_ptr(), b.data_ptr(), None, 0,
                                 acc.data_ptr(), s.cuda_stream) == 0
    assert lib.fftgb_residual_sq(None, b.data_ptr(), None, 5, acc.data_ptr(),
                                 s.cuda_stream) == -1
    del ctypes


def test_fused_poisson_step_in_cuda_graph(ag, cuda):
    """The loss + gradient step captured in one CUDA graph (the library's
    launches go to torch's capture stream) replays to the eager results."""
    import torch
    dims = (64, 64, 64)
    rho = torch.from_numpy(_fields(dims, 2, 9)).to(cuda).requires_grad_(True)
    phit = torch.from_numpy(_fields(dims, 2, 10)).to(cuda)

    def step():
        rho.grad = None
        loss = ag.poisson_loss_fused(rho, phit)
        loss.backward()
        return loss
    ref_loss = step().item()
    ref_grad = rho.grad.detach().clone()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(3):
            step()
    torch.cuda.current_stream().wait_stream(side)
    rho.grad = None
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        gl = step()
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    assert abs(gl.item() - ref_loss) <= 1e-6 * abs(ref_loss)
    assert orc.rel_l2(rho.grad.cpu().numpy(), ref_grad.cpu().numpy()) <= 1e-6

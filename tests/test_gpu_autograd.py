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

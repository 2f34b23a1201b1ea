"""torch.autograd binding of the library's transforms.

Forward runs ``fftgb_exec``; backward runs ``fftgb_exec_adjoint`` - the
hand-written adjoint path (conjugate-transpose DFT with the same scale):
adjoint(forward) = unnormalised inverse, adjoint(inverse) = forward.  With
PyTorch's convention for complex gradients (the conjugate Wirtinger
derivative), the gradient of y = A x is A^H applied to the incoming
gradient, which is exactly the adjoint.

The kernels compute in complex64; complex128 inputs (used by gradcheck) are
rounded to complex64 on the way in and widened on the way out.
"""
from __future__ import annotations

import torch

from .plan import Plan


class _FFTn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, plan: Plan, inverse: bool, scale: float):
        ctx.plan = plan
        ctx.inverse = inverse
        ctx.scale = scale
        ctx.dtype = x.dtype
        xc = x.detach().to(torch.complex64).contiguous()
        y = plan.execute(xc, inverse=inverse, scale=scale)
        return y.to(x.dtype) if x.dtype != torch.complex64 else y

    @staticmethod
    def backward(ctx, gy):
        g = gy.detach().to(torch.complex64).contiguous()
        gx = ctx.plan.execute(g, inverse=ctx.inverse, scale=ctx.scale,
                              adjoint=True)
        if ctx.dtype != torch.complex64:
            gx = gx.to(ctx.dtype)
        return gx, None, None, None


_PLANS: dict = {}


def plan_for(dims, batch: int) -> Plan:
    key = (tuple(dims), int(batch))
    p = _PLANS.get(key)
    if p is None:
        p = Plan(dims, batch)
        _PLANS[key] = p
    return p


def fftn(x: torch.Tensor, dims, inverse: bool = False, scale: float = 1.0,
         plan: Plan | None = None) -> torch.Tensor:
    """Differentiable batched C2C FFT over the trailing ``len(dims)`` axes of
    ``x`` (shape (..., *dims)), unnormalised unless ``scale`` says otherwise."""
    dims = tuple(int(d) for d in dims)
    n = 1
    for d in dims:
        n *= d
    if x.shape[-len(dims):] != dims:
        raise ValueError(f"trailing shape {tuple(x.shape[-len(dims):])} != {dims}")
    batch = x.numel() // n
    p = plan if plan is not None else plan_for(dims, batch)
    y = _FFTn.apply(x.reshape(-1), p, bool(inverse), float(scale))
    return y.reshape(x.shape)


def poisson_filter(dims):
    """G(k) = 1/|k|^2 with G(0) = 0 on an integer wavenumber grid (float32,
    shape dims), k = n * fftfreq(n) per axis."""
    ks = torch.meshgrid(*[torch.fft.fftfreq(d, d=1.0 / d) for d in dims],
                        indexing="ij")
    k2 = sum(k.double() ** 2 for k in ks)
    g = torch.where(k2 > 0, 1.0 / torch.where(k2 > 0, k2, torch.ones_like(k2)),
                    torch.zeros_like(k2))
    return g.float()


def poisson_loss(rho: torch.Tensor, phi_target: torch.Tensor,
                 g: torch.Tensor) -> torch.Tensor:
    """sum |IFFT3(FFT3(rho) * G) / N^3 - phi_target|^2 over a batch of grids
    (rho: (..., nz, ny, nx) complex)."""
    dims = tuple(g.shape)
    n = g.numel()
    rk = fftn(rho, dims)
    phi = fftn(rk * g.to(rk.device).to(rk.real.dtype), dims, inverse=True,
               scale=1.0 / n)
    return ((phi - phi_target).abs() ** 2).sum()

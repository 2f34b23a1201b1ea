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


class _PoissonLoss(torch.autograd.Function):
    """loss = sum |A rho - phi_t|^2 with A = IFFT3(G . FFT3(.)) / N^3 and
    G = 1/|k|^2 computed inside the transform kernels.

    forward:  g = G . F rho       (fftgb_exec_filtered: G in the last pass)
              phi = F^-1 g / N^3  (fftgb_exec, unnormalised inverse, scaled)
              r = phi - phi_t, loss = sum |r|^2 (fftgb_residual_sq, one pass)
    backward: A^H = F^H G (F^-1 / N^3)^H with the hand-written adjoints
              (adjoint(forward) = unnormalised inverse, adjoint(scaled
              inverse) = scaled forward), so
              h = G . adjoint(F^-1 / N^3) r  (fftgb_exec_adjoint_filtered)
              grad_rho = 2 adjoint(F) h        (fftgb_exec_adjoint)
              grad_phi_t = -2 r."""

    @staticmethod
    def forward(ctx, rho, phi_target, plan: Plan, n3: int):
        from . import _lib
        x = rho.detach().to(torch.complex64).contiguous().reshape(-1)
        t = phi_target.detach().to(torch.complex64).contiguous().reshape(-1)
        g = plan.execute(x, filter="poisson")
        phi = plan.execute(g, inverse=True, scale=1.0 / n3)
        r = torch.empty_like(phi)
        acc = torch.zeros(1, dtype=torch.float64, device=rho.device)
        s = torch.cuda.current_stream(rho.device)
        _lib.check(_lib.lib().fftgb_residual_sq(phi.data_ptr(), t.data_ptr(), r.data_ptr(),
                                                phi.numel(), acc.data_ptr(), s.cuda_stream),
                   "fftgb_residual_sq")
        ctx.plan = plan
        ctx.n3 = n3
        ctx.shape = rho.shape
        ctx.dtypes = (rho.dtype, phi_target.dtype)
        ctx.save_for_backward(r)
        return acc.to(torch.float32 if rho.dtype == torch.complex64 else torch.float64)[0]

    @staticmethod
    def backward(ctx, gout):
        (r,) = ctx.saved_tensors
        plan = ctx.plan
        grad_rho = grad_t = None
        if ctx.needs_input_grad[0]:
            h = plan.execute(r, inverse=True, scale=1.0 / ctx.n3, adjoint=True,
                             filter="poisson")
            gr = plan.execute(h, inverse=False, scale=2.0, adjoint=True)
            grad_rho = (gr * gout.to(gr.real.dtype)).reshape(ctx.shape).to(ctx.dtypes[0])
        if ctx.needs_input_grad[1]:
            grad_t = (r * (-2.0 * gout.to(r.real.dtype))).reshape(ctx.shape).to(ctx.dtypes[1])
        return grad_rho, grad_t, None, None


def poisson_loss_fused(rho: torch.Tensor, phi_target: torch.Tensor) -> torch.Tensor:
    """The loss of ``poisson_loss`` (trailing 3 axes of rho are the grid) with
    the filter inside the transform kernels and the residual and its sum of
    squares in one kernel; differentiable in rho and phi_target."""
    dims = tuple(int(d) for d in rho.shape[-3:])
    n3 = dims[0] * dims[1] * dims[2]
    batch = rho.numel() // n3
    if phi_target.shape != rho.shape:
        raise ValueError("rho and phi_target must have the same shape")
    return _PoissonLoss.apply(rho, phi_target, plan_for(dims, batch), n3)


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

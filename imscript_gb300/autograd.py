"""torch.autograd.Function over the converged Laplace/Poisson fill.

Forward: u = fill(g, f), the converged 5-point solve of the NaN pixels of g
with data term f (f = div G for a guidance field G, computed by the caller in
torch so that autograd carries the gradient on to G).

Backward: one adjoint solve A lambda = dL/du_U of the symmetric masked
operator, then dL/dg = dL/du + lambda scattered to the known 5-neighbours
(0 at the NaN pixels) and dL/df = -lambda at the unknowns (0 elsewhere).
Both directions go through the same C ABI (simpois_solve_device,
simpois_adjoint_device).
"""
from __future__ import annotations

import torch

from . import simpois as _sp


class SimpoisFill(torch.autograd.Function):
    @staticmethod
    def forward(ctx, g, f, rtol):
        out, reps = _sp.solve(g.detach(), None if f is None else f.detach(), tstep=0.25, rtol=rtol)
        ctx.save_for_backward(g)
        ctx.rtol = rtol
        ctx.has_f = f is not None
        ctx.reports = reps
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        gi, gd, _ = _sp.adjoint(grad_out, g.detach(), rtol=ctx.rtol,
                                want_dat=ctx.has_f and ctx.needs_input_grad[1])
        return (gi if ctx.needs_input_grad[0] else None,
                gd if (ctx.has_f and ctx.needs_input_grad[1]) else None,
                None)


def fill(g, f=None, rtol=1e-6):
    """Differentiable converged fill; g (pd,h,w) float32 CUDA with NaN holes."""
    return SimpoisFill.apply(g, f, rtol)


def divergence(gx, gy):
    """Backward-difference divergence of (gx, gy) with the clamped border,
    the data term whose Poisson fill reproduces a field whose forward-difference
    gradient is (gx, gy)."""
    f = gx.clone()
    f[..., :, 1:] = f[..., :, 1:] - gx[..., :, :-1]
    f = f + gy
    f[..., 1:, :] = f[..., 1:, :] - gy[..., :-1, :]
    return f

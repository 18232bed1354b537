"""``torch.autograd.Function`` for the EFF operator.

Forward: ``y = EFF(x, f)`` -- one fused kernel that transforms the
windowed patches and the PSFs, multiplies, inverse transforms and
overlap-adds, leaving both spectra behind.  Backward: one fused adjoint kernel computes both ``F^T g`` and
``X^T g`` from a single transform of the incoming gradient, reusing both
cached spectra (the two cnvtp calls of olaGPU.py:261-311 that blind
deconvolution needs: image step and PSF step).
"""
from __future__ import annotations

import torch

from .eff import EffPlan


class EFFFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, f, plan: EffPlan):
        batch = x.shape[0] if x.dim() == 3 else None
        fhat = plan.empty_spectrum(batch)
        xhat = plan.empty_spectrum(batch)
        y = plan.forward_both(x.detach(), f.detach(), xhat_out=xhat, fhat_out=fhat)
        ctx.plan = plan
        ctx.fhat = fhat
        ctx.xhat = xhat
        return y

    @staticmethod
    def backward(ctx, gy):
        need_x, need_f = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if not (need_x or need_f):
            return None, None, None
        gx, gf = ctx.plan.adjoint(gy.contiguous(), ctx.fhat if need_x else None,
                                  ctx.xhat if need_f else None, want_image=need_x, want_psf=need_f)
        return gx, gf, None


def eff(x: torch.Tensor, f: torch.Tensor, plan: EffPlan) -> torch.Tensor:
    """Differentiable ``y = EFF(x, f)`` on ``plan``'s geometry."""
    return EFFFunction.apply(x, f, plan)

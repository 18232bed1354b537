"""``torch.autograd.Function`` for the EFF operator.

Forward: ``y = EFF(x, f)`` -- one spectrum kernel for the PSFs, one fused
forward kernel for the image that also leaves the windowed-patch spectrum
behind.  Backward: one fused adjoint kernel computes both ``F^T g`` and
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
        fhat = plan.psf_spectrum(f.detach())
        xhat = plan.empty_spectrum(x.shape[0] if x.dim() == 3 else None)
        y = plan.forward_image(x.detach(), fhat, xhat_out=xhat)
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

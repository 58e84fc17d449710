"""torch.autograd binding of the cap forward operator (test binding).

CapOperator.apply(index, absorption, context, n, posspec) returns the cap
values S G(index + i absorption) as an (n, F, F, 2) float tensor; its
backward is the hand-written adjoint (tdm_adjoint), so a loss on the cap
values differentiates through the GPU kernels.  Tensors are CUDA float32,
contiguous; posspec is a (2n,) int32 tensor (x values then y values).
"""
from __future__ import annotations

import torch


class CapOperator(torch.autograd.Function):
    @staticmethod
    def forward(ctx, index, absorption, context, n, posspec):
        F = context.F
        caps = torch.empty((n, F, F, 2), dtype=torch.float32, device=index.device)
        context.forward(index.contiguous(), None if absorption is None else absorption.contiguous(), n=n,
                        posspec=posspec, caps_out=caps)
        context.synchronize()
        ctx.context, ctx.n, ctx.posspec = context, n, posspec
        ctx.has_absorption = absorption is not None
        return caps

    @staticmethod
    def backward(ctx, grad_caps):
        c = ctx.context
        D = c.D
        gi = torch.empty((D, D, D), dtype=torch.float32, device=grad_caps.device)
        ga = torch.empty_like(gi) if ctx.has_absorption else None
        c.adjoint(grad_caps.contiguous(), n=ctx.n, posspec=ctx.posspec, index_out=gi, absorption_out=ga)
        c.synchronize()
        return gi, ga, None, None, None


def cap_forward(index, absorption, context, n, posspec):
    """Differentiable S G(index + i absorption)."""
    return CapOperator.apply(index, absorption, context, n, posspec)

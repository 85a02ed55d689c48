"""torch.autograd wrapper of the DC-PSE apply over the C-ABI.

``dcpse_apply(f, pos, plan)`` returns ``[n_outputs, n]`` = L(pos) f (FP64,
batched outputs of the plan, weights assembled at ``pos`` with the plan's
neighbour list held fixed).  Its backward is the hand-written adjoint:
``dcpse_vjp_field`` (transposed stencil) for ``f`` and
``dcpse_vjp_positions`` (through every particle's moment-matrix solve) for
``pos``.  There is no automatic differentiation through the kernels.
"""
from __future__ import annotations

import torch

from . import _capi as C


class DcpseApply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, pos, plan, eps_fixed=None):
        plan.assemble(pos.detach(), C.ASSEMBLE_FAST | C.STORE_OUT_F64, eps_fixed=eps_fixed)
        y = plan.apply(f.detach(), C.F64)
        ctx.plan = plan
        ctx.eps_fixed = eps_fixed
        ctx.generation = plan.generation
        ctx.save_for_backward(f.detach(), pos.detach())
        return y

    @staticmethod
    def backward(ctx, gy):
        f, pos = ctx.saved_tensors
        plan = ctx.plan
        gy = gy.contiguous().to(torch.float64)
        # re-assemble only if the plan changed since forward (another
        # assembly, a new list) or eps was given (a tensor autograd does not
        # guard against in-place changes); pos itself is a saved tensor
        if plan.generation != ctx.generation or ctx.eps_fixed is not None:
            plan.assemble(pos, C.ASSEMBLE_FAST | C.STORE_OUT_F64, eps_fixed=ctx.eps_fixed)
        gf = plan.vjp_field(gy, C.F64) if ctx.needs_input_grad[0] else None
        gp = plan.vjp_positions(pos, f, gy, eps_fixed=ctx.eps_fixed) if ctx.needs_input_grad[1] else None
        return gf, gp, None, None


def dcpse_apply(f, pos, plan, eps_fixed=None):
    return DcpseApply.apply(f, pos, plan, eps_fixed)

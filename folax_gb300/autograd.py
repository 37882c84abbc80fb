"""torch.autograd.Function over the fused loss + adjoint (testing only).

forward returns mean_b L_b; backward returns the kernel's dLoss/dcontrol and
dLoss/ddofs scaled by the incoming gradient.  The gradients are computed in
the same launch as the loss, so backward does no extra GPU work.
"""
from __future__ import annotations

import torch


class FELossFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, fe_loss, control, dofs):
        mean, _, _, du, dc = fe_loss.ComputeBatchLossAndGrad(control, dofs)
        ctx.save_for_backward(du, dc)
        ctx.shapes = (control.shape, dofs.shape)
        return mean

    @staticmethod
    def backward(ctx, g):
        du, dc = ctx.saved_tensors
        cshape, ushape = ctx.shapes
        dc = dc if dc.shape == cshape else dc.sum(dim=0).reshape(cshape)
        return None, g * dc.reshape(cshape), g * du.reshape(ushape)


def fe_loss(fe_loss_obj, control, dofs):
    return FELossFunction.apply(fe_loss_obj, control, dofs)

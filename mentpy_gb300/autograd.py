"""Differentiable GPU sweep: ``torch.autograd.Function`` over the adjoint kernel.

mentpy has no automatic differentiation: training loops call finite
differences of whole simulations (mentpy/gradients/_finite_difference.py:9-25).
``sweep_states`` returns the batched output states as a differentiable
function of the angles; its backward is one launch of the adjoint kernel
(recompute-from-checkpoint reverse sweep), independent of the number of
angles.
"""
from __future__ import annotations

import torch

from .sweep import StatevectorSweep


class _SweepFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, angles, inputs, sweep):
        out, _status, _ = sweep.forward(angles.detach(), inputs, ref_phase=False)
        ctx.sweep = sweep
        ctx.inputs = inputs
        ctx.save_for_backward(angles)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (angles,) = ctx.saved_tensors
        g = ctx.sweep.adjoint(angles.detach(), ctx.inputs, grad_out.contiguous())
        return g.to(angles.dtype), None, None


def sweep_states(sweep: StatevectorSweep, angles: torch.Tensor, inputs=None) -> torch.Tensor:
    """Output states [B, 2^n_out] of ``sweep`` (no reference global phase),
    differentiable with respect to ``angles`` [B, A] (float64 or float32 CUDA
    tensor).  Gradients with respect to ``inputs`` are not provided."""
    if angles.dim() == 1:
        angles = angles.unsqueeze(0)
    return _SweepFunction.apply(angles, inputs, sweep)


def fidelity_loss(sweep: StatevectorSweep, angles, inputs, targets):
    """``1 - mean_j |<t_j|z(angles_v, psi_j)>|^2`` per angle vector with its
    gradient, fused in one kernel launch: returns ``(loss [V], grad [V, A])``."""
    return sweep.fidelity_grad(angles, inputs, targets)

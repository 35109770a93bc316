"""Validation-only ``torch.autograd.Function`` over the adjoint C ABI.

``rollout(adjoint, U0, theta, n_steps, dt0)`` returns the state after
``n_steps`` FP64 do_step calls as a CPU float64 tensor; its backward calls
``splash_adjoint_backward`` (checkpointed discrete adjoint on the GPU).  It
exists so that gradients of the rollout can be checked with torch tooling
next to finite differences and the tangent-linear model; it is not a
training path (states cross the host boundary at both ends).
"""
from __future__ import annotations

import numpy as np
import torch

from . import Adjoint


class SplashRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U0: torch.Tensor, theta: torch.Tensor, adjoint: Adjoint, n_steps: int, dt0: float):
        U0n = U0.detach().to("cpu", torch.float64).contiguous().numpy()
        thn = theta.detach().to("cpu", torch.float64).contiguous().numpy()
        Uf = adjoint.forward(U0n, thn, n_steps, dt0)
        adjoint._generation = getattr(adjoint, "_generation", 0) + 1
        ctx.adjoint = adjoint
        ctx.generation = adjoint._generation
        ctx.args = (U0n.copy(), thn.copy(), n_steps, dt0)
        return torch.from_numpy(Uf)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        adj: Adjoint = ctx.adjoint
        if getattr(adj, "_generation", None) != ctx.generation:
            # another rollout ran on this object since: redo this one's forward
            U0n, thn, n_steps, dt0 = ctx.args
            adj.forward(U0n, thn, n_steps, dt0)
            adj._generation = ctx.generation = adj._generation + 1
        lam = np.ascontiguousarray(grad_out.detach().to("cpu", torch.float64).numpy())
        gU, gth = adj.backward(lam)
        return torch.from_numpy(gU), torch.from_numpy(gth), None, None, None


def rollout(adjoint: Adjoint, U0: torch.Tensor, theta: torch.Tensor, n_steps: int, dt0: float) -> torch.Tensor:
    """State after n_steps FP64 steps, differentiable in U0 and theta."""
    return SplashRollout.apply(U0, theta, adjoint, n_steps, dt0)

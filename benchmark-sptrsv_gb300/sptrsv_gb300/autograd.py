"""Differentiable triangular solve: x = op(L)^-1 b as a torch.autograd.Function.

Forward runs the sync-free solve; backward runs the adjoint (transposed)
sync-free solve op(L)^T lambda = dLoss/dx on the same analysis in reverse
dependency order, and the same kernel forms dLoss/dL(i,j) = -lambda_i * x_j
on the stored pattern only. dLoss/db = lambda. x is kept from the forward pass;
with ``recompute=True`` (when memory is short) only b is kept and backward
solves for x again before the adjoint solve.
"""
from __future__ import annotations

import torch

from .solver import SyncFreeSolver


class SparseTriangularSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values: torch.Tensor, b: torch.Tensor, solver: SyncFreeSolver, recompute: bool = False):
        x = solver.solve(b, values=values)
        ctx.solver = solver
        ctx.values_version = values._version
        ctx.recompute = bool(recompute)
        # keep x, or (recompute) only b: x is solved for again in backward
        ctx.save_for_backward(values, b if ctx.recompute else x)
        return x

    @staticmethod
    def backward(ctx, gx: torch.Tensor):
        values, kept = ctx.saved_tensors
        solver: SyncFreeSolver = ctx.solver
        # the staged values are still the forward ones unless another call replaced them
        restage = solver.values is not values or values._version != ctx.values_version
        if ctx.recompute:
            x = solver.solve(kept, values=values if restage else None)
            restage = False  # the solve above staged them
        else:
            x = kept
        need_dval = ctx.needs_input_grad[0]
        lam, dval = solver.solve_adjoint(gx, x, values=values if restage else None, grad_values=need_dval)
        db = lam if ctx.needs_input_grad[1] else None
        return dval, db, None, None


def sparse_triangular_solve(solver: SyncFreeSolver, values: torch.Tensor, b: torch.Tensor,
                            recompute: bool = False) -> torch.Tensor:
    """x = op(L)^-1 b with L = (solver's pattern, ``values``); differentiable in values and b.
    ``recompute=True`` keeps b instead of x for the backward pass and solves again there."""
    return SparseTriangularSolve.apply(values, b, solver, recompute)

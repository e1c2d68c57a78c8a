"""Wiring of the autograd Function on the CPU: a stand-in solver with the
SyncFreeSolver methods the Function calls (dense FP64 triangular solves) lets
torch.autograd.gradcheck check the backward pass -- adjoint solve, pattern-only
value gradient, restaging, and the recompute mode -- without a GPU. The CUDA
path itself is checked against finite differences in test_gpu_adjoint.py."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from sptrsv_gb300 import matgen
from sptrsv_gb300.autograd import sparse_triangular_solve


class DenseStandIn:
    """SyncFreeSolver's solve / solve_adjoint contract on CPU tensors (CSC pattern)."""

    def __init__(self, m):
        self.n = m.n
        self.lower = m.lower
        self.rows = torch.from_numpy(m.row_idx.astype(np.int64))
        cols = np.repeat(np.arange(m.n), np.diff(m.col_ptr))
        self.cols = torch.from_numpy(cols.astype(np.int64))
        self.values = None
        self.solves = 0

    def _dense(self):
        L = torch.zeros(self.n, self.n, dtype=self.values.dtype)
        L[self.rows, self.cols] = self.values
        return L

    def solve(self, b, values=None):
        if values is not None:
            self.values = values
        self.solves += 1
        B = b.reshape(self.n, -1)
        x = torch.linalg.solve_triangular(self._dense(), B, upper=not self.lower)
        return x.reshape(b.shape)

    def solve_adjoint(self, g, x=None, values=None, grad_values=False):
        if values is not None:
            self.values = values
        G = g.reshape(self.n, -1)
        lam = torch.linalg.solve_triangular(self._dense().T, G, upper=self.lower)
        dval = None
        if grad_values:
            X = x.reshape(self.n, -1)
            dval = -(lam[self.rows] * X[self.cols]).sum(dim=1)
        return lam.reshape(g.shape), dval


@pytest.mark.parametrize("lower", [True, False])
@pytest.mark.parametrize("recompute", [False, True])
@pytest.mark.parametrize("rhs", [1, 3])
def test_gradcheck_through_the_function(lower, recompute, rhs):
    m = matgen.poisson_band(12, 3.0, 6, seed=7, lower=lower)
    solver = DenseStandIn(m)
    values = torch.from_numpy(m.val.copy()).requires_grad_(True)
    shape = (m.n,) if rhs == 1 else (m.n, rhs)
    b = torch.randn(shape, dtype=torch.float64, generator=torch.Generator().manual_seed(rhs)).requires_grad_(True)
    assert torch.autograd.gradcheck(lambda v, bb: sparse_triangular_solve(solver, v, bb, recompute=recompute),
                                    (values, b), eps=1e-6, atol=1e-8)


def test_recompute_keeps_b_and_solves_again():
    m = matgen.poisson_band(10, 3.0, 5, seed=3)
    solver = DenseStandIn(m)
    values = torch.from_numpy(m.val.copy()).requires_grad_(True)
    b = torch.randn(m.n, dtype=torch.float64, generator=torch.Generator().manual_seed(0)).requires_grad_(True)
    w = torch.randn(m.n, dtype=torch.float64, generator=torch.Generator().manual_seed(1))
    grads = {}
    for recompute in (False, True):
        solver.solves = 0
        x = sparse_triangular_solve(solver, values, b, recompute=recompute)
        (w * x).sum().backward()
        grads[recompute] = (values.grad.clone(), b.grad.clone())
        assert solver.solves == (2 if recompute else 1)
        values.grad = None
        b.grad = None
    assert torch.allclose(grads[False][0], grads[True][0], rtol=1e-13, atol=0)
    assert torch.allclose(grads[False][1], grads[True][1], rtol=1e-13, atol=0)

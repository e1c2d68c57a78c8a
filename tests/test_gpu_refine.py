"""FP32 storage/solve + FP64-residual iterative refinement: forward error against
the FP64 oracle must be at most 1e-10 (relative, max norm)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

TOL_FWD = 1e-10


def relerr(x, ref):
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("schedule", [1, 2, 3])
def test_refined_forward_error(cuda, name, schedule):
    from sptrsv_gb300 import SyncFreeSolver
    g = load_golden(name)
    n, rhs = int(g["n"]), int(g["rhs"])
    sub = 0 if int(g["lower"]) else 1
    s = SyncFreeSolver(g["col_ptr"], g["row_idx"], n, sub, values=g["val"], schedule=schedule)
    b = cuda.from_numpy(g["b"].reshape(n, rhs)).cuda()
    x, iters, est = s.solve_refine(b)
    assert 1 <= iters <= 4
    assert est <= 1e-12
    assert relerr(x.cpu().numpy(), g["x64"]) <= TOL_FWD


@pytest.mark.parametrize("rhs", [1, 16, 64])
def test_refine_column_major_1m_like(cuda, oracle_port, rhs):
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.poisson_band(20_000, 9.0, 2000, seed=2)
    B = np.random.default_rng(rhs).standard_normal((m.n, rhs))
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, B)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val)
    b_cm = cuda.from_numpy(np.ascontiguousarray(B.T)).cuda().t()
    x, iters, est = s.solve_refine(b_cm)
    if rhs > 1:
        assert x.stride() == (1, m.n)
    assert relerr(x.cpu().numpy(), ref) <= TOL_FWD
    # fixed-step mode (no read-back) gives the same answer after the same number of steps
    x2, it2, _ = s.solve_refine(b_cm, tol=0.0, max_iter=iters)
    assert relerr(x2.cpu().numpy(), ref) <= TOL_FWD


def test_refine_reports_non_convergence(cuda):
    from sptrsv_gb300 import SptrsvError, SyncFreeSolver, _lib, matgen
    m = matgen.poisson_band(3000, 6.0, 300, seed=4)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val)
    b = cuda.ones(m.n, dtype=cuda.float64, device="cuda")
    with pytest.raises(SptrsvError) as ei:
        s.solve_refine(b, tol=1e-300, max_iter=1)
    assert ei.value.status == _lib.ERR_NOT_CONVERGED

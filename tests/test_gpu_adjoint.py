"""Adjoint (transposed) solve, fused value gradient, and the autograd Function,
checked against the oracle's gradient (transposition + serial executor with the
opposite substitution) and central finite differences. Tolerances: 1e-12
relative (max norm) in FP64; the exact adjoint is bit-identical to the serial
executor run on the transposed CSC."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu


def relerr(x, ref):
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("cfg", [dict(lanes=1), dict(lanes=4, order_block=1), dict(lanes=32, order_block=10**9),
                                 dict(exact=True), dict(exact=True, order_block=10**9, chunk=64),
                                 dict(staged=False, lanes=1), dict(staged=False, exact=True),
                                 dict(chunk=16, stage_entries=40), dict(chunk=16, stage_entries=40, exact=True),
                                 dict(fused_grad=1), dict(fused_grad=1, staged=False, lanes=4),
                                 dict(staged=False, warp_sync=True, fused_grad=1),
                                 dict(staged=False, warp_sync=True, exact=True, order_block=64, chunk=64),
                                 dict(staged=False, warp_sync=True, order_block=128, chunk=128),
                                 dict(staged=False, warp_sync=True, split=4),
                                 dict(staged=False, warp_sync=True, split=0),
                                 dict(staged=False, warp_sync=True, split=4, wsync_batch=1),
                                 dict(staged=False, warp_sync=True, split=0, wsync_batch=2, order_block=128,
                                      chunk=128)],
                         ids=lambda c: "-".join(f"{k}{v}" for k, v in c.items()))
def test_adjoint_and_gradient_vs_oracle(cuda, name, cfg):
    from oracle import oracle
    from sptrsv_gb300 import SyncFreeSolver
    g = load_golden(name)
    n, rhs = int(g["n"]), int(g["rhs"])
    sub = 0 if int(g["lower"]) else 1
    w = np.random.default_rng(n + rhs).standard_normal((n, rhs))
    x = g["x64"].reshape(n, rhs)
    lam_ref, dval_ref = oracle.adjoint_gradient(g["col_ptr"], g["row_idx"], g["val"], n, sub, x, w)
    s = SyncFreeSolver(g["col_ptr"], g["row_idx"], n, sub, values=g["val"], schedule=2, **cfg)
    lam, dval = s.solve_adjoint(cuda.from_numpy(w).cuda(), cuda.from_numpy(x).cuda(), grad_values=True)
    lam = lam.cpu().numpy()
    if cfg.get("exact"):
        assert np.array_equal(lam.ravel().view(np.uint64), lam_ref.ravel().view(np.uint64))
    else:
        assert relerr(lam, lam_ref) <= 1e-12
    assert relerr(dval.cpu().numpy(), dval_ref) <= 1e-12
    dval2 = s.grad_values(cuda.from_numpy(lam).cuda(), cuda.from_numpy(x).cuda())
    assert relerr(dval2.cpu().numpy(), dval_ref) <= 1e-12


@pytest.mark.parametrize("lower", [True, False])
@pytest.mark.parametrize("rhs", [1, 3, 8])
def test_autograd_against_finite_differences(cuda, lower, rhs):
    from sptrsv_gb300 import SyncFreeSolver, matgen, sparse_triangular_solve
    m = matgen.poisson_band(400, 5.0, 80, seed=rhs, lower=lower)
    rng = np.random.default_rng(rhs)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution)
    val = cuda.tensor(m.val, device="cuda", requires_grad=True)
    b = cuda.tensor(rng.standard_normal((m.n, rhs)), device="cuda", requires_grad=True)
    wt = cuda.tensor(rng.standard_normal((m.n, rhs)), device="cuda")
    x = sparse_triangular_solve(s, val, b)
    loss = (wt * x).sum()
    loss.backward()
    gv, gb = val.grad.cpu().numpy(), b.grad.cpu().numpy()

    def f(vv, bb):
        with cuda.no_grad():
            return float((wt * s.solve(bb, values=vv)).sum())

    h = 1e-6
    v0, b0 = val.detach().clone(), b.detach().clone()
    for e in rng.choice(m.nnz, 32, replace=False):
        vp, vm = v0.clone(), v0.clone()
        vp[e] += h
        vm[e] -= h
        fd = (f(vp, b0) - f(vm, b0)) / (2 * h)
        assert abs(fd - gv[e]) <= 1e-6 * max(1.0, abs(fd))
    for _ in range(32):
        i, k = int(rng.integers(m.n)), int(rng.integers(rhs))
        bp, bm = b0.clone(), b0.clone()
        bp[i, k] += h
        bm[i, k] -= h
        fd = (f(v0, bp) - f(v0, bm)) / (2 * h)
        assert abs(fd - gb[i, k]) <= 1e-6 * max(1.0, abs(fd))


def test_autograd_column_major_and_fp32(cuda):
    from oracle import oracle
    from sptrsv_gb300 import SyncFreeSolver, matgen, sparse_triangular_solve
    m = matgen.poisson_band(2000, 6.0, 300, seed=5, lower=False)
    rng = np.random.default_rng(5)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution)
    b_np = rng.standard_normal((m.n, 4))
    w_np = rng.standard_normal((m.n, 4))
    b = cuda.from_numpy(np.ascontiguousarray(b_np.T)).cuda().t().requires_grad_(True)   # column-major
    val = cuda.tensor(m.val, device="cuda", requires_grad=True)
    x = sparse_triangular_solve(s, val, b)
    (cuda.from_numpy(w_np).cuda() * x).sum().backward()
    x_ref = oracle.port().solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b_np)
    lam_ref, dval_ref = oracle.adjoint_gradient(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, x_ref, w_np)
    assert relerr(b.grad.cpu().numpy(), lam_ref) <= 1e-12
    assert relerr(val.grad.cpu().numpy(), dval_ref) <= 1e-12
    # FP32 storage: same gradients to FP32 accuracy
    b32 = cuda.from_numpy(b_np.astype(np.float32)).cuda().requires_grad_(True)
    v32 = cuda.tensor(m.val.astype(np.float32), device="cuda", requires_grad=True)
    x32 = sparse_triangular_solve(s, v32, b32)
    (cuda.from_numpy(w_np.astype(np.float32)).cuda() * x32).sum().backward()
    assert relerr(b32.grad.cpu().numpy(), lam_ref) <= 1e-5
    assert relerr(v32.grad.cpu().numpy(), dval_ref) <= 1e-4

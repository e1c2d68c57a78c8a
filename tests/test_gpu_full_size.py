"""Parity at the benchmark workloads' full sizes, through the C ABI, against the
FP64 oracle (the serial executor restated from
SpTRSV_cuda/sptrsv_syncfree_serialref.h:25-108) run on the same seeded inputs.

Workloads (the same generators and seeds the benchmark uses):
  * 10k-row Poisson(8) band system, rhs 1;
  * the 4,194,304-row power-law triangle, forward and backward (rhs 1);
  * the 1,000,000-row band system at rhs 1, 16 and 64, column-major B ~ N(0,1),
    plain FP64 and FP32 + FP64-residual refinement;
  * all 512 uneven batch systems (half lower, half upper), rhs 4, one batched
    launch (FP64 and refined), each system against its own oracle solve;
  * the 1M-row system at rhs 8: adjoint gradients w.r.t. b and the stored
    values against the oracle gradient (transposition + serial solve,
    tranpose.h:6-43) and against central differences (h = 1e-6) on 64 random
    entries of each.

Tolerances (relative, max norm): FP64 solves 1e-12; exact mode bit-identical;
refined solves 1e-10; gradients 1e-12 against the oracle gradient; central
differences |fd - g| <= 1e-6 * max(1, |fd|)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL_REFINE = 1e-10


def relerr(x, ref):
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


def _col_major(cuda, a):
    """Device copy of the n x k array `a` stored column-major (a transposed view)."""
    return cuda.from_numpy(np.ascontiguousarray(a.T)).cuda().t()


# ------------------------------------------------------------------ 10k-row system
def test_system_10k(cuda, oracle_port):
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.system_10k()
    assert (m.n, m.substitution) == (10_000, 0)
    b = m.matvec(np.ones(m.n))
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, 0, b)
    bd = cuda.from_numpy(b).cuda()
    for kw in (dict(), dict(schedule=1), dict(schedule=3), dict(schedule=2, staged=True)):
        s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, 0, values=m.val, **kw)
        assert relerr(s.solve(bd).cpu().numpy(), ref) <= TOL64, kw
        s.close()
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, 0, values=m.val, schedule=2, exact=True)
    x = s.solve(bd).cpu().numpy()
    assert np.array_equal(x.view(np.uint64), ref.view(np.uint64))
    s.close()


# ------------------------------------------------------------------ power-law 4M system
@pytest.fixture(scope="module")
def powerlaw():
    from sptrsv_gb300 import matgen
    lo = matgen.system_powerlaw_4m(seed=1, lower=True)
    return {"fwd": lo, "bwd": lo.transpose()}


@pytest.mark.parametrize("direction", ["fwd", "bwd"])
def test_powerlaw_4m(cuda, oracle_port, powerlaw, direction):
    from sptrsv_gb300 import SyncFreeSolver
    m = powerlaw[direction]
    assert m.n == 4_194_304
    rng = np.random.default_rng(11)
    for b in (m.matvec(np.ones(m.n)), rng.standard_normal(m.n)):
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
        bd = cuda.from_numpy(b).cuda()
        s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val)
        assert relerr(s.solve(bd).cpu().numpy(), ref) <= TOL64
        s.close()
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, schedule=2, exact=True)
    x = s.solve(bd).cpu().numpy()
    assert np.array_equal(x.view(np.uint64), ref.view(np.uint64))
    s.close()


# ------------------------------------------------------------------ 1M system, many right-hand sides
@pytest.fixture(scope="module")
def system_1m():
    from sptrsv_gb300 import matgen
    return matgen.system_1m(seed=2)


@pytest.mark.parametrize("rhs", [1, 16, 64])
def test_system_1m_multi_rhs(cuda, oracle_port, system_1m, rhs):
    from sptrsv_gb300 import SyncFreeSolver
    m = system_1m
    assert m.n == 1_000_000
    B = np.random.default_rng(rhs).standard_normal((m.n, rhs))
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, B if rhs > 1 else B[:, 0])
    ref = ref.reshape(m.n, rhs)
    b = _col_major(cuda, B)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val)
    x = s.solve(b)
    if rhs > 1:
        assert x.stride() == b.stride()       # column-major in, column-major out
    assert relerr(x.cpu().numpy(), ref) <= TOL64
    xr, iters, est = s.solve_refine(b, tol=1e-12)
    assert relerr(xr.cpu().numpy(), ref) <= TOL_REFINE
    assert iters >= 1
    s.close()


# ------------------------------------------------------------------ 512 uneven systems in one launch
@pytest.fixture(scope="module")
def batch512():
    from sptrsv_gb300 import matgen
    return matgen.batch_uneven(count=512, seed=3)


def test_batch_512_every_system(cuda, oracle_port, batch512):
    from sptrsv_gb300 import SyncFreeSolver
    systems = batch512
    assert len(systems) == 512
    assert sum(m.substitution for m in systems) == 256
    rhs = 4
    rng = np.random.default_rng(4)
    bs = [rng.standard_normal((m.n, rhs)) for m in systems]
    vals = np.concatenate([m.val for m in systems])
    s = SyncFreeSolver(batch=[(m.col_ptr, m.row_idx, m.n, m.substitution) for m in systems], values=vals)
    b = cuda.from_numpy(np.concatenate(bs)).cuda()
    x64 = s.solve(b).cpu().numpy()
    xr, iters, est = s.solve_refine(b, tol=1e-12)
    xr = xr.cpu().numpy()
    worst64 = worst_r = 0.0
    for k, m in enumerate(systems):
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, bs[k])
        sl = slice(s.offsets[k], s.offsets[k + 1])
        e64, er = relerr(x64[sl], ref), relerr(xr[sl], ref)
        assert e64 <= TOL64, f"system {k} (n={m.n}, FP64): {e64:.3e}"
        assert er <= TOL_REFINE, f"system {k} (n={m.n}, refined): {er:.3e}"
        worst64, worst_r = max(worst64, e64), max(worst_r, er)
    s.close()


# ------------------------------------------------------------------ adjoint on the 1M system, rhs 8
def test_adjoint_1m_rhs8(cuda, system_1m):
    from oracle import oracle
    from sptrsv_gb300 import SyncFreeSolver, sparse_triangular_solve
    m = system_1m
    rhs = 8
    rng = np.random.default_rng(4)
    B = rng.standard_normal((m.n, rhs))
    W = rng.standard_normal((m.n, rhs))
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution)
    val = cuda.from_numpy(m.val).cuda().requires_grad_(True)
    b = cuda.from_numpy(B).cuda().requires_grad_(True)
    w = cuda.from_numpy(W).cuda()
    x = sparse_triangular_solve(s, val, b)
    (w * x).sum().backward()
    gb, gv = b.grad.cpu().numpy(), val.grad.cpu().numpy()
    # the oracle gradient: x from the serial executor, lambda from the serial
    # executor on the transposed CSC
    x_ref = oracle.port().solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, B)
    assert relerr(x.detach().cpu().numpy(), x_ref) <= TOL64
    lam_ref, dval_ref = oracle.adjoint_gradient(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, x_ref, W)
    assert relerr(gb, lam_ref) <= TOL64
    assert relerr(gv, dval_ref) <= TOL64
    # central differences, h = 1e-6, evaluated with the deterministic (exact-order)
    # executor; the loss difference is summed over the solution difference
    fdsolver = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, schedule=2, exact=True)
    h = 1e-6
    v0 = cuda.from_numpy(m.val).cuda()
    b0 = cuda.from_numpy(B).cuda()

    def dloss(vp, bp, vm, bm):
        with cuda.no_grad():
            return float((w * (fdsolver.solve(bp, values=vp) - fdsolver.solve(bm, values=vm))).sum()) / (2 * h)

    for e in rng.choice(m.nnz, 64, replace=False):
        vp, vm = v0.clone(), v0.clone()
        vp[int(e)] += h
        vm[int(e)] -= h
        fd = dloss(vp, b0, vm, b0)
        assert abs(fd - gv[e]) <= 1e-6 * max(1.0, abs(fd)), f"value entry {e}: fd {fd} vs {gv[e]}"
    for _ in range(64):
        i, k = int(rng.integers(m.n)), int(rng.integers(rhs))
        bp, bm = b0.clone(), b0.clone()
        bp[i, k] += h
        bm[i, k] -= h
        fd = dloss(v0, bp, v0, bm)
        assert abs(fd - gb[i, k]) <= 1e-6 * max(1.0, abs(fd)), f"b[{i},{k}]: fd {fd} vs {gb[i, k]}"
    fdsolver.close()
    s.close()

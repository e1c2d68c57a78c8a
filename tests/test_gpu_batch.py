"""Batched solve: many independent lower and upper triangles of uneven sizes
analysed into one handle and solved in one persistent launch. Each system's
slice is checked against the oracle run on that system alone (1e-12 relative
in FP64, bit-identical in exact mode, 1e-10 after mixed-precision refinement)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def relerr(x, ref):
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


@pytest.fixture(scope="module")
def systems():
    from sptrsv_gb300 import matgen
    sys_ = matgen.batch_uneven(count=14, seed=3, nmin=50, nmax=6000)
    sys_.append(matgen.laplace2d_lower(20, lower=False))
    sys_.append(matgen.star(300))
    sys_.append(matgen.diagonal(7, lower=False))
    return sys_


def _solver(systems, **kw):
    from sptrsv_gb300 import SyncFreeSolver
    vals = np.concatenate([m.val for m in systems])
    return SyncFreeSolver(batch=[(m.col_ptr, m.row_idx, m.n, m.substitution) for m in systems], values=vals, **kw)


@pytest.mark.parametrize("cfg", [dict(), dict(order_block=10**9), dict(chunk=64, order_block=64),
                                 dict(schedule=1), dict(schedule=3), dict(staged=False, lanes=4),
                                 dict(chunk=40, stage_entries=40, stages=3),
                                 dict(staged=False, warp_sync=True), dict(staged=False, warp_sync=True,
                                                                          order_block=256, chunk=256),
                                 dict(staged=False, warp_sync=True, split=4),
                                 dict(staged=False, warp_sync=True, order_block=512, chunk=512, block=64,
                                      import_deps=True),
                                 dict(staged=False, warp_sync=True, order_block=100, chunk=100, block=128,
                                      wsync_batch=1)],
                         ids=lambda c: "-".join(f"{k}{v}" for k, v in c.items()) or "default")
@pytest.mark.parametrize("rhs", [1, 4])
def test_batch_matches_per_system_oracle(cuda, oracle_port, systems, cfg, rhs):
    s = _solver(systems, **cfg)
    assert s.n == sum(m.n for m in systems)
    rng = np.random.default_rng(rhs)
    bs = [rng.standard_normal((m.n, rhs)) for m in systems]
    x = s.solve(cuda.from_numpy(np.concatenate(bs)).cuda()).cpu().numpy()
    for k, m in enumerate(systems):
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, bs[k])
        assert relerr(x[s.offsets[k]:s.offsets[k + 1]], ref) <= 1e-12, f"system {k}"


def test_batch_exact_and_refine(cuda, oracle_port, systems):
    s = _solver(systems, exact=True)
    rng = np.random.default_rng(9)
    bs = [rng.standard_normal((m.n, 4)) for m in systems]
    b = np.concatenate(bs)
    x = s.solve(cuda.from_numpy(b).cuda()).cpu().numpy()
    refs = [oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, bs[k]) for k, m in enumerate(systems)]
    for k in range(len(systems)):
        xs = np.ascontiguousarray(x[s.offsets[k]:s.offsets[k + 1]])
        assert np.array_equal(xs.view(np.uint64), refs[k].view(np.uint64)), f"system {k}"
    s2 = _solver(systems)
    bc = cuda.from_numpy(np.ascontiguousarray(b.T)).cuda().t()   # column-major [n, 4]
    xr, iters, est = s2.solve_refine(bc)
    xr = xr.cpu().numpy()
    for k in range(len(systems)):
        assert relerr(xr[s2.offsets[k]:s2.offsets[k + 1]], refs[k]) <= 1e-10


def test_batch_rejects_bad_members(cuda):
    from sptrsv_gb300 import SptrsvError, SyncFreeSolver, _lib
    good = (np.array([0, 2, 3]), np.array([0, 1, 1]), 2, 0)
    duplicate = (np.array([0, 1, 3]), np.array([0, 1, 1]), 2, 0)     # row 1 twice in column 1
    upper_as_lower = (np.array([0, 1, 3]), np.array([0, 0, 1]), 2, 0)
    bad_row = (np.array([0, 2, 3]), np.array([0, 5, 1]), 2, 0)       # local row outside its system
    short_ptr = (np.array([0, 2, 2]), np.array([0, 1, 1]), 2, 0)     # last pointer != nnz of the member
    for bad in (duplicate, upper_as_lower, bad_row, short_ptr):
        with pytest.raises(SptrsvError) as ei:
            SyncFreeSolver(batch=[good, bad])
        assert ei.value.status == _lib.ERR_BAD_STRUCTURE
    s = SyncFreeSolver(batch=[good, good], values=np.ones(6))
    x = s.solve(cuda.ones(4, dtype=cuda.float64, device="cuda")).cpu().numpy()
    np.testing.assert_allclose(x, [1, 0, 1, 0])

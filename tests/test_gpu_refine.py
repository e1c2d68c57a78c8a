"""FP32 storage/solve + FP64-residual iterative refinement: forward error against
the FP64 oracle must be at most 1e-10 (relative, max norm). The fused first step
runs with the residual in FP64 (fused_refine=1) or in double-float on the FP32
pipe (fused_refine=2); both are held to the same tolerance."""
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
@pytest.mark.parametrize("schedule,fused", [(0, 1), (0, 2), (0, 0), (1, 1), (2, 1), (2, 2), (2, 0), (3, 1)])
def test_refined_forward_error(cuda, name, schedule, fused):
    from sptrsv_gb300 import SyncFreeSolver
    g = load_golden(name)
    n, rhs = int(g["n"]), int(g["rhs"])
    sub = 0 if int(g["lower"]) else 1
    s = SyncFreeSolver(g["col_ptr"], g["row_idx"], n, sub, values=g["val"], schedule=schedule,
                       fused_refine=fused)
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


def _fused_cases():
    from sptrsv_gb300 import matgen
    return {
        "band_fwd": lambda: matgen.poisson_band(30_000, 9.0, 3000, seed=11),
        "band_bwd": lambda: matgen.poisson_band(30_000, 9.0, 3000, seed=12, lower=False),
        "powerlaw_fwd": lambda: matgen.system_powerlaw_4m(seed=1, n=60_000, target_nnz=600_000),
        "powerlaw_bwd": lambda: matgen.system_powerlaw_4m(seed=1, n=60_000, target_nnz=600_000).transpose(),
        # deep and narrow: the automatic plan picks a blocked layout
        "laplace_fwd": lambda: matgen.laplace2d_lower(300),
        "laplace_bwd": lambda: matgen.laplace2d_lower(300).transpose(),
    }


@pytest.mark.parametrize("case", list(_fused_cases()))
@pytest.mark.parametrize("rhs", [1, 3, 16, 64])
def test_fused_first_step_against_oracle(cuda, oracle_port, case, rhs):
    """The fused pass (FP32 solve, FP64 residual and FP32 correction in one walk of
    the DAG) reaches the 1e-10 forward error in its single step on these diagonally
    dominant systems, like the separate passes do, for row- and column-major blocks."""
    from sptrsv_gb300 import SyncFreeSolver
    m = _fused_cases()[case]()
    B = np.random.default_rng(rhs).standard_normal((m.n, rhs))
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, B)
    results = {}
    for fused in (1, 2, 0):
        s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, fused_refine=fused)
        for layout in ("row", "col"):
            b = cuda.from_numpy(B).cuda()
            if layout == "col":
                b = cuda.from_numpy(np.ascontiguousarray(B.T)).cuda().t()
            x, iters, est = s.solve_refine(b, tol=1e-12)
            assert relerr(x.cpu().numpy(), ref) <= TOL_FWD, (fused, layout)
            assert 1 <= iters <= 3 and est <= 1e-12
            # fixed-step mode: no read-back, same result after the same number of steps
            x2, it2, _ = s.solve_refine(b, tol=0.0, max_iter=iters)
            assert it2 == iters
            assert relerr(x2.cpu().numpy(), ref) <= TOL_FWD
            results[(fused, layout)] = (x.cpu().numpy(), iters)
        s.close()
    assert results[(1, "row")][1] == 1 and results[(2, "row")][1] == 1
    # the fused steps (FP64 or double-float residual) and the separate passes agree
    # to well below the tolerance
    assert relerr(results[(1, "row")][0], results[(0, "row")][0]) <= TOL_FWD
    assert relerr(results[(2, "row")][0], results[(0, "row")][0]) <= TOL_FWD


def test_fused_refine_more_steps_and_option(cuda, oracle_port):
    """max_iter > 1 continues with separate passes after the fused step; the option
    round-trips and 0 selects the separate passes."""
    from sptrsv_gb300 import SyncFreeSolver, _lib, matgen
    m = matgen.poisson_band(8000, 8.0, 800, seed=13)
    B = np.random.default_rng(3).standard_normal((m.n, 2))
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, 0, B)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, 0, values=m.val)
    assert s.get_option(_lib.OPTION_FUSED_REFINE) == 2
    b = cuda.from_numpy(B).cuda()
    for steps in (1, 2, 3):
        x, it, _ = s.solve_refine(b, tol=0.0, max_iter=steps)
        assert it == steps
        assert relerr(x.cpu().numpy(), ref) <= TOL_FWD
    for mode in (0, 1):
        s.set_option(_lib.OPTION_FUSED_REFINE, mode)
        assert s.get_option(_lib.OPTION_FUSED_REFINE) == mode
        for steps in (1, 2):
            x, it, _ = s.solve_refine(b, tol=0.0, max_iter=steps)
            assert relerr(x.cpu().numpy(), ref) <= TOL_FWD
        x, it, _ = s.solve_refine(b)
        assert relerr(x.cpu().numpy(), ref) <= TOL_FWD
    # re-staged values reach the double-float weights too
    s.set_values(cuda.from_numpy(2.0 * m.val).cuda())
    x, it, _ = s.solve_refine(b, tol=0.0, max_iter=1)
    assert relerr(x.cpu().numpy(), ref / 2.0) <= TOL_FWD


@pytest.mark.parametrize("case", ["one", "diagonal", "chain", "dense64", "star"])
def test_fused_refine_edge_structures(cuda, oracle_port, case):
    """Edge structures through the fused pass: a single unknown, no dependencies at
    all, a chain (one unknown per level), a dense triangle (one long list per row)
    and a star (one unknown feeding all others)."""
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = {"one": lambda: matgen.diagonal(1), "diagonal": lambda: matgen.diagonal(5000),
         "chain": lambda: matgen.chain(3000), "dense64": lambda: matgen.dense_lower(64),
         "star": lambda: matgen.star(4000)}[case]()
    for rhs in (1, 5):
        B = np.random.default_rng(rhs).standard_normal((m.n, rhs))
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, B)
        for fused in (1, 2):
            s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, fused_refine=fused)
            x, iters, est = s.solve_refine(cuda.from_numpy(B).cuda())
            assert relerr(x.cpu().numpy(), ref) <= TOL_FWD, (case, rhs, fused)
            s.close()


@pytest.mark.parametrize("lower", [True, False])
def test_fused_refine_on_blocked_layout_with_importer(cuda, oracle_port, lower):
    """On a deep, narrow mesh the automatic plan picks a blocked layout; the fused
    double-float step then runs with an importer warp per block. Same tolerance as
    every refined solve, with the importer on and off."""
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.laplace2d_lower(600, lower=lower)
    b_h = np.random.default_rng(7).standard_normal(m.n)
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b_h)
    b = cuda.from_numpy(b_h).cuda()
    for imp in (True, False):
        s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, import_deps=imp)
        assert s.info()["order_block"] < m.n
        for _ in range(2):
            x, iters, est = s.solve_refine(b, tol=1e-12)
            assert iters == 1 and est <= 1e-12
            assert relerr(x.cpu().numpy(), ref) <= TOL_FWD, imp
        s.close()

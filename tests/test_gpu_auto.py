"""The automatic executor plan (SPTRSV_SCHED_AUTO): what it picks from the
analysis and that every path it picks matches the oracle (FP64, <= 1e-12
relative in the max norm)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def relerr(x, ref):
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


def _solver(m, **kw):
    from sptrsv_gb300 import SyncFreeSolver
    return SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, **kw)


@pytest.mark.parametrize("lower", [True, False])
def test_local_deep_dag_gets_blocked_order(cuda, oracle_port, lower):
    from sptrsv_gb300 import matgen
    m = matgen.laplace2d_lower(200, lower=lower)          # 399 levels, 100 unknowns per level
    s = _solver(m)
    inf = s.info()
    assert inf["nlevels"] == 399
    blk = 32 * -(-m.n // inf["nlevels"])                  # 32 level widths
    assert inf["order_block"] == blk and inf["chunk"] == blk and inf["warp_sync"] == 1 and inf["staged"] == 0
    assert inf["locality_permille"] >= 960
    for rhs in (1, 4, 16):
        b = np.random.default_rng(rhs).standard_normal((m.n, rhs))
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
        x = s.solve(cuda.from_numpy(b).cuda()).cpu().numpy()
        assert relerr(x, ref) <= TOL64
    # the transposed solve walks the blocked layout in reverse
    g = np.random.default_rng(7).standard_normal(m.n)
    t = m.transpose()
    ref = oracle_port.solve(t.col_ptr, t.row_idx, t.val, t.n, t.substitution, g)
    lam, _ = s.solve_adjoint(cuda.from_numpy(g).cuda())
    lam = lam.cpu().numpy()
    assert relerr(lam, ref) <= TOL64


@pytest.mark.parametrize("band, blocked", [(100, True), (2000, False)])
def test_blocked_order_follows_the_locality_threshold(cuda, oracle_port, band, blocked):
    """Blocked orders only where >= 96 % of the dependencies stay inside the blocks:
    a 160k-row band of width 100 with two entries per column (97.5 % local) is
    blocked; the same with width 2000 (92.5 % local, where a blocked order
    measured 4.8x slower) stays in global level order."""
    from sptrsv_gb300 import matgen
    m = matgen.poisson_band(160_000, 2.0, band, seed=11)
    s = _solver(m)
    inf = s.info()
    assert inf["nlevels"] >= 256
    assert (inf["locality_permille"] >= 960) == blocked
    assert (inf["order_block"] < m.n) == blocked
    b = np.random.default_rng(band).standard_normal(m.n)
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
    assert relerr(s.solve(cuda.from_numpy(b).cuda()).cpu().numpy(), ref) <= TOL64


def test_dependencies_per_iteration_follow_co_arrival(cuda, oracle_port):
    """One dependency per lockstep iteration unless at least half of the unknowns
    have two or more dependencies on the level just before their own (the mesh
    triangle: both neighbours sit one level up and land together); lists
    averaging more than 3 entries take one; an explicit option wins."""
    from sptrsv_gb300 import matgen
    cases = [(matgen.laplace2d_lower(200), {}, 2), (matgen.poisson_band(40_000, 2.0, 300, seed=21), {}, 1),
             (matgen.chain(5000), {}, 1), (matgen.poisson_band(20_000, 9.0, 400, seed=22), {}, 1),
             (matgen.laplace2d_lower(200), {"wsync_batch": 4}, 4)]
    for m, kw, want in cases:
        s = _solver(m, **kw)
        inf = s.info()
        assert inf["wsync_batch"] == want, (m.n, kw, inf)
        if (m.nnz - m.n) > 3 * m.n:
            assert inf["coarrive_permille"] == 0
        elif not kw:
            assert (inf["coarrive_permille"] >= 500) == (want == 2)
        b = np.random.default_rng(m.n).standard_normal(m.n)
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
        assert relerr(s.solve(cuda.from_numpy(b).cuda()).cpu().numpy(), ref) <= TOL64
        s.close()


@pytest.mark.parametrize("which", ["mesh", "band", "random"])
def test_coarrival_count_matches_the_oracle_levels(cuda, oracle_port, which):
    """sptrsv_info.coarrive_permille against a count over the oracle's level sets
    (findlevel.h:6-69): unknowns with two or more dependencies on the level just
    before their own, per mille of the unknowns with any dependency."""
    from sptrsv_gb300 import matgen
    m = {"mesh": lambda: matgen.laplace2d_lower(120, lower=False),
         "band": lambda: matgen.poisson_band(30_000, 2.0, 300, seed=23),
         "random": lambda: matgen.random_small(3000, 0.002, seed=3)}[which]()
    assert m.nnz - m.n <= 3 * m.n
    nl, level_ptr, level_item = oracle_port.findlevel(m.col_ptr, m.row_idx, m.n)
    level = np.empty(m.n, dtype=np.int64)
    for lv in range(nl):
        level[level_item[level_ptr[lv]:level_ptr[lv + 1]]] = lv
    col = np.repeat(np.arange(m.n), np.diff(m.col_ptr))
    off = m.row_idx != col
    rows, deps = m.row_idx[off], col[off]                  # row depends on column
    prev = np.bincount(rows, weights=(level[deps] == level[rows] - 1), minlength=m.n)
    anyd = np.bincount(rows, minlength=m.n) > 0
    want = int(np.sum(prev >= 2) / np.sum(anyd) * 1000.0 + 0.5)
    s = _solver(m)
    assert s.info()["coarrive_permille"] == want
    s.close()


def test_wide_dag_stays_in_level_order(cuda, oracle_port):
    from sptrsv_gb300 import matgen
    m = matgen.poisson_band(20_000, 9.0, 4000, seed=5)     # dependencies spread over 4000 rows
    s = _solver(m)
    inf = s.info()
    assert inf["order_block"] >= m.n and inf["chunk"] == 256 and inf["block"] == 256 and inf["warp_sync"] == 1
    b = np.random.default_rng(1).standard_normal(m.n)
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
    assert relerr(s.solve(cuda.from_numpy(b).cuda()).cpu().numpy(), ref) <= TOL64


def test_long_lists_get_split(cuda, oracle_port):
    from sptrsv_gb300 import matgen
    m = matgen.power_law_band(30_000, 300_000, 3000, seed=3, lower=False)   # long rows in the upper triangle
    s = _solver(m)
    assert s.info()["split"] == 32
    b = np.random.default_rng(2).standard_normal(m.n)
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
    assert relerr(s.solve(cuda.from_numpy(b).cuda()).cpu().numpy(), ref) <= TOL64


def test_uniformly_long_lists_stay_on_one_lane(cuda, oracle_port):
    """Lists that are long but alike (a band with ~40 entries per row) are not split:
    splitting pays only when a few lists are far longer than the rest."""
    from sptrsv_gb300 import matgen
    m = matgen.poisson_band(40_000, 40.0, 800, seed=6)
    s = _solver(m)
    assert s.info()["split"] == 0
    b = np.random.default_rng(3).standard_normal(m.n)
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
    assert relerr(s.solve(cuda.from_numpy(b).cuda()).cpu().numpy(), ref) <= TOL64


def test_explicit_options_override_the_plan(cuda, oracle_port):
    from sptrsv_gb300 import _lib, matgen
    m = matgen.laplace2d_lower(200)
    s = _solver(m, order_block=10**9, staged=True)
    inf = s.info()
    assert inf["order_block"] >= m.n and inf["staged"] == 1
    s2 = _solver(m, schedule=2)                              # explicit schedule: no plan at all
    assert s2.info()["warp_sync"] == 0
    b = np.random.default_rng(3).standard_normal(m.n)
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
    for solver in (s, s2):
        assert relerr(solver.solve(cuda.from_numpy(b).cuda()).cpu().numpy(), ref) <= TOL64
    assert s.get_option(_lib.OPTION_SCHEDULE) == 0

"""CUDA-graph capture of the solve path and the autotuner."""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def relerr(x, ref):
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


@pytest.mark.parametrize("schedule", [1, 2, 3])
def test_graph_replay_matches_eager(cuda, schedule):
    from sptrsv_gb300 import SyncFreeSolver
    g = load_golden("uneven3000_bwd")
    n, rhs = int(g["n"]), int(g["rhs"])
    s = SyncFreeSolver(g["col_ptr"], g["row_idx"], n, 1, values=g["val"], schedule=schedule)
    b = cuda.from_numpy(g["b"].reshape(n, rhs)).cuda()
    x = cuda.empty_like(b)
    graph = s.graph(b, x, kind=0, count=3)
    x.zero_()
    graph.replay()
    s.check()
    assert relerr(x.cpu().numpy(), g["x64"]) <= 1e-12
    b.mul_(2.0)            # the graph reads b in place
    graph.replay()
    s.check()
    assert relerr(x.cpu().numpy(), 2 * g["x64"]) <= 1e-12


def test_refine_graph(cuda, oracle_port):
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.poisson_band(5000, 8.0, 500, seed=8)
    B = np.random.default_rng(1).standard_normal((m.n, 8))
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, 0, B)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, 0, values=m.val)
    b = cuda.from_numpy(B).cuda()
    x = cuda.empty_like(b)
    graph = s.graph(b, x, kind=1, count=2)
    x.zero_()
    graph.replay()
    s.check()
    assert relerr(x.cpu().numpy(), ref) <= 1e-10


@pytest.mark.parametrize("rhs", [1, 4])
def test_tune_picks_a_working_configuration(cuda, oracle_port, rhs):
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.poisson_band(20_000, 8.0, 2000, seed=rhs, lower=False)
    B = np.random.default_rng(rhs).standard_normal((m.n, rhs))
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, 1, B)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, 1)
    b = cuda.from_numpy(B).cuda()
    res = s.tune(b, values=cuda.from_numpy(m.val).cuda(), reps=2)
    assert res["best_ms"] > 0
    assert relerr(s.solve(b).cpu().numpy(), ref) <= 1e-12
    # the chosen options round-trip through JSON into a fresh handle
    opts = json.loads(json.dumps(s.tuned_options()))
    s2 = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, 1, values=m.val)
    s2.apply_options(opts)
    assert s2.tuned_options() == opts
    assert relerr(s2.solve(b).cpu().numpy(), ref) <= 1e-12


@pytest.mark.parametrize("opt", [1, 2, 3])
@pytest.mark.parametrize("rhs", [3, 20, 40])
def test_push_schedule_reference_lane_modes(cuda, oracle_port, opt, rhs):
    """The push schedule (the reference's scheme) with the reference's lane modes:
    entries (1), right-hand sides (2) and the per-column rule (3), on a triangle with
    short and long columns (so the rule picks both modes), forward and backward."""
    from sptrsv_gb300 import SyncFreeSolver, matgen
    lo = matgen.power_law_band(6000, 60_000, 3000, seed=17)
    for m in (lo, lo.transpose()):
        B = np.random.default_rng(rhs).standard_normal((m.n, rhs))
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, B)
        s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, schedule=1, opt=opt)
        assert s.get_option(22) == opt
        assert relerr(s.solve(cuda.from_numpy(B).cuda()).cpu().numpy(), ref) <= 1e-12
        s.close()


@pytest.mark.parametrize("tile", [1, 2, 4])
@pytest.mark.parametrize("rhs", [5, 16, 64])
def test_pull_rhs_tile(cuda, oracle_port, tile, rhs):
    """Right-hand sides per lane of the warp-synchronous many-rhs executor, row- and
    column-major blocks, forward and backward."""
    from sptrsv_gb300 import SyncFreeSolver, matgen
    lo = matgen.poisson_band(8000, 7.0, 900, seed=rhs)
    for m in (lo, lo.transpose()):
        B = np.random.default_rng(tile).standard_normal((m.n, rhs))
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, B)
        s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, rhs_tile=tile)
        assert relerr(s.solve(cuda.from_numpy(B).cuda()).cpu().numpy(), ref) <= 1e-12
        bc = cuda.from_numpy(np.ascontiguousarray(B.T)).cuda().t()
        assert relerr(s.solve(bc).cpu().numpy(), ref) <= 1e-12
        s.close()


@pytest.mark.parametrize("case", ["mesh_600", "band_30k"])
@pytest.mark.parametrize("rhs", [1, 8])
def test_tune_on_non_benchmark_systems(cuda, oracle_port, case, rhs):
    """The tuner on systems other than the benchmark's (a 600 x 600 mesh, whose order
    blocks derive from its own level widths, and a band), one and eight right-hand
    sides: its pick solves to the oracle, and every tuned axis round-trips."""
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.laplace2d_lower(600) if case == "mesh_600" else matgen.poisson_band(30_000, 5.0, 700, seed=4)
    B = np.random.default_rng(rhs).standard_normal((m.n, rhs))
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, B)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution)
    b = cuda.from_numpy(B).cuda()
    res = s.tune(b, values=cuda.from_numpy(m.val).cuda(), reps=2)
    assert res["best_ms"] > 0
    opts = s.tuned_options()
    for key in ("smem_tier", "opt", "rhs_tile", "order_block"):
        assert key in opts
    assert relerr(s.solve(b).cpu().numpy(), ref) <= 1e-12
    s2 = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val)
    s2.apply_options(opts)
    assert relerr(s2.solve(b).cpu().numpy(), ref) <= 1e-12

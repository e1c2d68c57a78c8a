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

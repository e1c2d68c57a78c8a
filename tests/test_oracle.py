"""The CPU oracle (oracle/sptrsv_oracle.c) pinned against the reference's own
outputs: golden fixtures made by tests/golden/make_golden.py from the
reference's serial code, plus live comparisons where the reference build exists."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_names, load_golden


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_reference_golden(name, oracle_port):
    g = load_golden(name)
    n, rhs = int(g["n"]), int(g["rhs"])
    sub = 0 if int(g["lower"]) else 1
    deg = oracle_port.analyser(g["row_idx"], n)
    np.testing.assert_array_equal(deg, g["in_degree"])
    x64 = oracle_port.executor(g["col_ptr"], g["row_idx"], g["val"], deg, n, sub, rhs, g["b"])
    assert np.array_equal(x64.view(np.uint64), g["x64"].view(np.uint64)), "FP64 executor not bit-identical"
    x32 = oracle_port.executor(g["col_ptr"], g["row_idx"], g["val"].astype(np.float32), deg, n, sub, rhs,
                               g["b"].astype(np.float32))
    assert np.array_equal(x32.view(np.uint32), g["x32"].view(np.uint32)), "FP32 executor not bit-identical"
    rp, ci, cv = oracle_port.transpose(g["col_ptr"], g["row_idx"], g["val"], n)
    np.testing.assert_array_equal(rp, g["csr_ptr"])
    np.testing.assert_array_equal(ci, g["csr_idx"])
    np.testing.assert_array_equal(cv, g["csr_val"])
    nl, lp, li = oracle_port.findlevel(g["col_ptr"], g["row_idx"], n)
    assert nl == int(g["nlevel"])
    np.testing.assert_array_equal(lp, g["level_ptr"])
    np.testing.assert_array_equal(li, g["level_item"])
    assert tuple(oracle_port.findlevel_csc(g["col_ptr"], g["row_idx"], n)) == tuple(int(v) for v in g["level_stats"])


def test_hand_case_solves_exactly(oracle_port):
    g = load_golden("hand4_fwd")
    x = oracle_port.solve(g["col_ptr"], g["row_idx"], g["val"], 4, 0, g["b"])
    np.testing.assert_array_equal(x, [1.0, 2.0, 3.0, 4.0])
    nl, lp, _ = oracle_port.findlevel(g["col_ptr"], g["row_idx"], 4)
    assert nl == 4 and list(lp) == [0, 1, 2, 3, 4]


def test_manufactured_solution_check(oracle_port):
    """The reference's own acceptance test: L1-relative error below 1e-4 (serialref.h:194-209)."""
    from oracle import oracle
    for name in ("unitrand_band1500_fwd", "unitrand_band1500_bwd", "band2000_fwd", "laplace24_bwd"):
        g = load_golden(name)
        assert oracle.l1_rel_err(g["x64"], g["x_true"]) < 1e-4


def _gen():
    from sptrsv_gb300 import matgen
    yield matgen.poisson_band(20_000, 8.0, 2000, seed=21)
    yield matgen.poisson_band(20_000, 8.0, 2000, seed=22, lower=False)
    yield matgen.laplace2d_lower(60, lower=False)
    yield matgen.power_law_band(30_000, 250_000, 5000, seed=23)


def test_port_matches_live_reference_build(oracle_port):
    from oracle import oracle
    ref = oracle.ref()
    if ref is None:
        pytest.skip("reference checkout not available on this host")
    rng = np.random.default_rng(5)
    for m in _gen():
        for rhs in (1, 2):
            b = rng.standard_normal(m.n * rhs)
            deg_p = oracle_port.analyser(m.row_idx, m.n)
            np.testing.assert_array_equal(deg_p, ref.analyser(m.row_idx, m.n))
            xp = oracle_port.executor(m.col_ptr, m.row_idx, m.val, deg_p, m.n, m.substitution, rhs, b)
            xr = ref.executor(m.col_ptr, m.row_idx, m.val, deg_p, m.n, m.substitution, rhs, b)
            assert np.array_equal(xp.view(np.uint64), xr.view(np.uint64))
        nl_p = oracle_port.findlevel(m.col_ptr, m.row_idx, m.n)
        nl_r = ref.findlevel(m.col_ptr, m.row_idx, m.n)
        assert nl_p[0] == nl_r[0]
        np.testing.assert_array_equal(nl_p[1], nl_r[1])
        np.testing.assert_array_equal(nl_p[2], nl_r[2])
        assert oracle_port.findlevel_csc(m.col_ptr, m.row_idx, m.n) == ref.findlevel_csc(m.col_ptr, m.row_idx, m.n)


def test_port_agrees_with_scipy(oracle_port):
    from scipy.sparse.linalg import spsolve_triangular
    from sptrsv_gb300 import matgen
    for m in (matgen.poisson_band(5000, 8.0, 500, seed=3), matgen.poisson_band(5000, 8.0, 500, seed=4, lower=False)):
        b = np.random.default_rng(1).standard_normal(m.n)
        x = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
        xs = spsolve_triangular(m.to_scipy().tocsr(), b, lower=m.lower)
        assert np.max(np.abs(x - xs)) <= 1e-12 * np.max(np.abs(xs))


def test_adjoint_gradient_matches_finite_differences():
    from oracle import oracle
    from sptrsv_gb300 import matgen
    m = matgen.poisson_band(300, 4.0, 60, seed=9)
    rng = np.random.default_rng(2)
    b = rng.standard_normal((m.n, 2))
    w = rng.standard_normal((m.n, 2))
    imp = oracle.port()

    def loss(val, bb):
        x = imp.solve(m.col_ptr, m.row_idx, val, m.n, m.substitution, bb)
        return float((w * x).sum())

    x = imp.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
    db, dval = oracle.adjoint_gradient(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, x, w)
    h = 1e-6
    for e in rng.choice(m.nnz, 16, replace=False):
        vp, vm = m.val.copy(), m.val.copy()
        vp[e] += h
        vm[e] -= h
        fd = (loss(vp, b) - loss(vm, b)) / (2 * h)
        assert abs(fd - dval[e]) <= 1e-6 * max(1.0, abs(fd))
    for i in rng.choice(m.n, 8, replace=False):
        bp, bm = b.copy(), b.copy()
        bp[i, 1] += h
        bm[i, 1] -= h
        fd = (loss(m.val, bp) - loss(m.val, bm)) / (2 * h)
        assert abs(fd - db[i, 1]) <= 1e-6 * max(1.0, abs(fd))


def test_malformed_input_is_reported_not_hung(oracle_port):
    """An in-degree that the executor can never satisfy is reported (the reference would spin)."""
    from oracle import oracle
    g = load_golden("band2000_fwd")
    n = int(g["n"])
    deg = oracle_port.analyser(g["row_idx"], n)
    deg[n // 2] += 1
    lib = oracle_port.lib
    import ctypes
    x = np.zeros(n)
    rc = lib.oracle_executor_f64(*(a.ctypes.data_as(ctypes.c_void_p) for a in (g["col_ptr"], g["row_idx"], g["val"], deg)),
                                 ctypes.c_int(n), ctypes.c_int(n), ctypes.c_int(0), ctypes.c_int(1),
                                 g["b"].ctypes.data_as(ctypes.c_void_p), x.ctypes.data_as(ctypes.c_void_p))
    assert rc == 1

"""Synthetic generators: storage invariants the reference expects (main.cu:212-237)."""
from __future__ import annotations

import numpy as np
import pytest

from sptrsv_gb300 import matgen


def _check(m):
    cp = m.col_ptr.astype(np.int64)
    assert cp[0] == 0 and cp[-1] == m.nnz and np.all(np.diff(cp) >= 1)
    ri = m.row_idx.astype(np.int64)
    assert ri.min() >= 0 and ri.max() < m.n
    diag = cp[:-1] if m.lower else cp[1:] - 1
    np.testing.assert_array_equal(ri[diag], np.arange(m.n))
    col = np.repeat(np.arange(m.n), np.diff(cp))
    assert np.all(ri >= col) if m.lower else np.all(ri <= col)
    same = col[1:] == col[:-1]
    assert np.all(ri[1:][same] > ri[:-1][same])
    a = m.to_scipy()
    off = abs(a - __import__("scipy").sparse.diags(a.diagonal()))
    d = np.abs(a.diagonal())
    assert np.all(d > np.asarray(off.sum(axis=0)).ravel()) and np.all(d > np.asarray(off.sum(axis=1)).ravel())


@pytest.mark.parametrize("make", [
    lambda: matgen.system_10k(),
    lambda: matgen.poisson_band(5000, 9.0, 700, seed=2, lower=False),
    lambda: matgen.power_law_band(50_000, 400_000, 5000, seed=1),
    lambda: matgen.random_small(400, 0.05, seed=3),
    lambda: matgen.dense_lower(40),
    lambda: matgen.star(50, lower=False),
    lambda: matgen.chain(100),
    lambda: matgen.diagonal(10),
])
def test_generator_invariants(make):
    _check(make())


def test_laplace_counts_and_levels():
    from oracle import oracle
    m = matgen.laplace2d_lower(30)
    assert m.n == 900 and m.nnz == 900 + 2 * 30 * 29
    assert oracle.port().findlevel_csc(m.col_ptr, m.row_idx, m.n)[0] == 2 * 30 - 1
    u = matgen.laplace2d_lower(30, lower=False)
    assert oracle.port().findlevel_csc(u.col_ptr, u.row_idx, u.n)[0] == 2 * 30 - 1


def test_10k_system_shape():
    m = matgen.system_10k()
    assert m.n == 10_000
    assert 85_000 < m.nnz < 95_000    # ~Poisson(8) off-diagonals + the diagonal
    assert np.array_equal(m.col_ptr, matgen.system_10k().col_ptr)  # seeded


def test_batch_uneven_small():
    sys_ = matgen.batch_uneven(count=8, seed=3, nmin=100, nmax=2000)
    assert len(sys_) == 8
    assert [s.lower for s in sys_] == [True, False] * 4
    for s in sys_:
        _check(s)

"""Input preparation with the reference's semantics (main.cu:142-358) on small files."""
from __future__ import annotations

import numpy as np
import pytest

from sptrsv_gb300 import mtx


def _write(tmp_path, text, name="a.mtx"):
    p = tmp_path / name
    p.write_text(text)
    return p


def test_general_real_and_extraction(tmp_path, oracle_port):
    p = _write(tmp_path, """%%MatrixMarket matrix coordinate real general
% comment
4 4 7
1 1 2.0
2 1 -1.0
3 2 4.5
4 1 1.0
4 3 3.0
1 4 9.0
3 3 1.0
""")
    m, n, rp, ci, v = mtx.read_mtx(p)
    assert (m, n) == (4, 4) and rp[-1] == 7
    L = mtx.extract_triangle(m, n, rp, ci, 0, seed=1)
    # strictly lower entries kept: (2,1),(3,2),(4,1),(4,3) + unit diagonal
    assert L.nnz == 4 + 4 and L.lower
    d = L.to_scipy().toarray()
    np.testing.assert_array_equal(np.diag(d), np.ones(4))
    assert np.all(np.triu(d, 1) == 0)
    assert set(np.unique(d[np.tril_indices(4, -1)][d[np.tril_indices(4, -1)] != 0])) <= set(range(1, 11))
    U = mtx.extract_triangle(m, n, rp, ci, 1, seed=1)
    assert U.nnz == 1 + 4 and not U.lower       # only (1,4) above the diagonal
    assert U.row_idx[U.col_ptr[-1] - 1] == 3     # diagonal closes the last column
    # manufactured solution solves back exactly with the serial oracle (reference check < 1e-4)
    x_ref, b = mtx.manufactured_rhs(L, rhs=2, seed=3)
    x = oracle_port.solve(L.col_ptr, L.row_idx, L.val, L.n, 0, b)
    from oracle import oracle
    assert oracle.l1_rel_err(x, x_ref) < 1e-12


def test_symmetric_pattern_expansion(tmp_path):
    p = _write(tmp_path, """%%MatrixMarket matrix coordinate pattern symmetric
3 3 3
1 1
2 1
3 2
""")
    m, n, rp, ci, v = mtx.read_mtx(p)
    assert rp[-1] == 5            # (1,1), (2,1), (1,2), (3,2), (2,3)
    np.testing.assert_array_equal(v, np.ones(5))


def test_csc_reader(tmp_path):
    # 3x3 lower: col 0 rows {0,1,2}, col 1 rows {1}, col 2 rows {2}; 1-based in the file
    p = _write(tmp_path, "3 3 5\n1 4 5 6\n1 2 3 2 3\n", name="l.csc")
    L = mtx.read_csc(p, 0, seed=2)
    np.testing.assert_array_equal(L.col_ptr, [0, 3, 4, 5])
    np.testing.assert_array_equal(L.row_idx, [0, 1, 2, 1, 2])
    assert np.all((L.val >= 1) & (L.val <= 10))


def test_rejects_non_square_and_bad_files(tmp_path):
    p = _write(tmp_path, "%%MatrixMarket matrix coordinate real general\n2 3 1\n1 1 1.0\n")
    m, n, rp, ci, v = mtx.read_mtx(p)
    with pytest.raises(ValueError):
        mtx.extract_triangle(m, n, rp, ci, 0)
    with pytest.raises(ValueError):
        mtx.read_mtx(_write(tmp_path, "not a matrix\n", name="b.mtx"))
    with pytest.raises(ValueError):
        mtx.read_mtx(_write(tmp_path, "%%MatrixMarket matrix coordinate real general\n2 2 2\n1 1 1.0\n", name="c.mtx"))

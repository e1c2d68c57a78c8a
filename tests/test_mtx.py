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


# ------------------------------------------------------------------ pinned against the reference's reader
def _mtx_goldens():
    from conftest import GOLDEN
    return sorted((GOLDEN / "mtx").glob("*.mtx"))


def _sorted_rows(row_ptr, col_idx, val):
    """CSR with every row's entries ordered by column (values carried along)."""
    ci, v = np.array(col_idx), np.array(val, dtype=np.float64)
    for r in range(len(row_ptr) - 1):
        a, b = row_ptr[r], row_ptr[r + 1]
        o = np.argsort(ci[a:b], kind="stable")
        ci[a:b], v[a:b] = ci[a:b][o], v[a:b][o]
    return ci, v


@pytest.mark.parametrize("path", _mtx_goldens(), ids=lambda p: p.stem)
def test_reader_matches_reference_reader(path):
    """read_mtx gives the CSR of the reference's reader (mmio_highlevel.h:137-296), up to
    the order of entries inside a row (the fixtures hold no duplicates)."""
    g = np.load(path.with_suffix(".npz"))
    m, n, rp, ci, v = mtx.read_mtx(path)
    assert (m, n) == (int(g["m"]), int(g["n"]))
    np.testing.assert_array_equal(rp, g["csr_ptr"])
    gci, gv = _sorted_rows(g["csr_ptr"], g["csr_idx"], g["csr_val"])
    np.testing.assert_array_equal(ci, gci)
    np.testing.assert_array_equal(v, gv)


@pytest.mark.parametrize("path", _mtx_goldens(), ids=lambda p: p.stem)
@pytest.mark.parametrize("substitution", [0, 1])
def test_extraction_matches_reference_pattern(path, substitution):
    """extract_triangle keeps the pattern main.cu:153-218 builds: strict triangle plus a
    unit diagonal, CSC with ascending rows (the reference's transposition)."""
    g = np.load(path.with_suffix(".npz"))
    m, n, rp, ci, v = mtx.read_mtx(path)
    t = mtx.extract_triangle(m, n, rp, ci, substitution, seed=7)
    key = "lower" if substitution == 0 else "upper"
    np.testing.assert_array_equal(t.col_ptr, g[f"{key}_col_ptr"])
    np.testing.assert_array_equal(t.row_idx, g[f"{key}_row_idx"])
    dpos = t.col_ptr[:-1] if substitution == 0 else t.col_ptr[1:] - 1
    np.testing.assert_array_equal(t.row_idx[dpos], np.arange(n))
    np.testing.assert_array_equal(t.val[dpos], np.ones(n))


def test_reader_against_live_reference_build(tmp_path):
    """Where the reference build exists: the live reader agrees on a larger seeded file,
    and on a file with a duplicated entry (which the reference keeps twice and read_mtx
    sums: the same matrix)."""
    from oracle import oracle
    if oracle.ref() is None:
        pytest.skip("reference checkout not available on this host")
    p = tmp_path / "band.mtx"
    write_band_mtx(p, 1500, 6, seed=8)
    ref = oracle.ref_read_mtx(p)
    m, n, rp, ci, v = mtx.read_mtx(p)
    np.testing.assert_array_equal(rp, ref[2])
    gci, gv = _sorted_rows(ref[2], ref[3], ref[4])
    np.testing.assert_array_equal(ci, gci)
    np.testing.assert_array_equal(v, gv)
    d = _write(tmp_path, "%%MatrixMarket matrix coordinate real general\n3 3 4\n1 1 1.0\n2 1 0.5\n2 1 0.25\n"
                         "3 3 2.0\n", name="dup.mtx")
    ref = oracle.ref_read_mtx(d)
    m, n, rp, ci, v = mtx.read_mtx(d)
    assert ref[2][-1] == 4 and rp[-1] == 3
    import scipy.sparse as sp
    a_ref = sp.csr_matrix((ref[4], ref[3], ref[2]), shape=(3, 3)).toarray()
    np.testing.assert_array_equal(sp.csr_matrix((v, ci, rp), shape=(3, 3)).toarray(), a_ref)


def write_band_mtx(path, n: int, per_row: int, seed: int, symmetric: bool = False):
    """A seeded general (or symmetric, lower storage) real band matrix, entries shuffled."""
    rng = np.random.default_rng(seed)
    rows, cols = [], []
    for r in range(n):
        lo, hi = max(0, r - 200), (r + 1 if symmetric else min(n, r + 200))
        cs = np.unique(rng.integers(lo, hi, size=per_row))
        rows += [r] * cs.size
        cols += cs.tolist()
    order = rng.permutation(len(rows))
    vals = rng.uniform(-1, 1, len(rows))
    kind = "symmetric" if symmetric else "general"
    lines = [f"%%MatrixMarket matrix coordinate real {kind}", f"{n} {n} {len(rows)}"]
    lines += [f"{rows[i] + 1} {cols[i] + 1} {vals[i]:.17g}" for i in order]
    path.write_text("\n".join(lines) + "\n")

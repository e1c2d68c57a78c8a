"""Input preparation with the reference's semantics.

* ``read_mtx``: a Matrix Market coordinate file (real / integer / pattern /
  complex-real-part) to CSR, as the reader of SpTRSV_cuda/mmio_highlevel.h:8-134
  and :137-296 builds it: symmetric and hermitian storage expanded (the mirror
  entry gets the same value), every other symmetry kind -- skew-symmetric
  included -- read as stored. Two deliberate differences, neither of which
  changes a solve: rows come out with ascending columns (the reference keeps
  file order; the triangle's CSC is sorted by both), and duplicate entries are
  summed (the reference keeps both copies, and its solvers add both).
* ``extract_triangle``: the reference's -forward / -backward preparation
  (SpTRSV_cuda/main.cu:153-218): keep the strictly lower (forward) or strictly
  upper (backward) part of A, give every kept entry a value rand()%10+1 (here:
  a seeded generator, integers 1..10), append a unit diagonal to every row,
  transpose to CSC (rows ascending inside each column, as the reference's
  transposition scatter produces them).
* ``read_csc``: the reference's -csc file (main.cu:247-294): ``m n nnz``, then
  n+1 one-based column pointers and nnz one-based row indices; values
  rand()%10+1 (seeded). Unlike the reference (which sorts each column with a
  call that has no effect), the structure is validated when it is analysed.
* ``manufactured_rhs``: x_ref with entries rand()%10+1 (seeded) and b = L x_ref
  in row-major n x rhs (main.cu:333-358).
"""
from __future__ import annotations

import numpy as np

from .matgen import CscTriangle


def read_mtx(path) -> tuple[int, int, np.ndarray, np.ndarray, np.ndarray]:
    """Returns (m, n, row_ptr, col_idx, val) of the CSR matrix in the file."""
    with open(path, "r") as f:
        header = f.readline().strip().split()
        if len(header) < 5 or header[0].lower() != "%%matrixmarket":
            raise ValueError(f"{path}: not a Matrix Market file")
        obj, fmt, field, sym = (h.lower() for h in header[1:5])
        if obj != "matrix" or fmt != "coordinate":
            raise ValueError(f"{path}: only coordinate matrices are supported")
        if field not in ("real", "integer", "pattern", "complex", "double"):
            raise ValueError(f"{path}: unsupported field {field}")
        line = f.readline()
        while line.startswith("%") or not line.strip():
            line = f.readline()
        m, n, nnz = (int(v) for v in line.split()[:3])
        data = np.loadtxt(f, ndmin=2) if nnz > 0 else np.zeros((0, 3))
    if data.shape[0] != nnz:
        raise ValueError(f"{path}: expected {nnz} entries, found {data.shape[0]}")
    rows = data[:, 0].astype(np.int64) - 1
    cols = data[:, 1].astype(np.int64) - 1
    if field == "pattern":
        vals = np.ones(nnz)
    else:
        vals = data[:, 2].astype(np.float64)   # complex: the real part
    if rows.size and (rows.min() < 0 or rows.max() >= m or cols.min() < 0 or cols.max() >= n):
        raise ValueError(f"{path}: index out of range")
    if sym in ("symmetric", "hermitian"):   # mmio_highlevel.h:175-178 (mm_is_symmetric || mm_is_hermitian)
        off = rows != cols
        rows, cols, vals = (np.concatenate([rows, cols[off]]), np.concatenate([cols, rows[off]]),
                            np.concatenate([vals, vals[off]]))
    import scipy.sparse as sp
    a = sp.coo_matrix((vals, (rows, cols)), shape=(m, n)).tocsr()
    a.sum_duplicates()
    a.sort_indices()
    return m, n, a.indptr.astype(np.int64), a.indices.astype(np.int32), a.data


def extract_triangle(m: int, n: int, row_ptr, col_idx, substitution: int, seed: int = 0) -> CscTriangle:
    """Strictly lower (substitution 0) or upper (1) part of A with values 1..10 and a unit
    diagonal, as CSC. main.cu:153-218."""
    if m != n:
        raise ValueError("the matrix is not square")
    rng = np.random.default_rng(seed)
    row_ptr = np.asarray(row_ptr, dtype=np.int64)
    col_idx = np.asarray(col_idx, dtype=np.int64)
    rows = np.repeat(np.arange(m, dtype=np.int64), np.diff(row_ptr))
    keep = col_idx < rows if substitution == 0 else col_idx > rows
    r, c = rows[keep], col_idx[keep]
    v = rng.integers(1, 11, size=r.size).astype(np.float64)
    d = np.arange(n, dtype=np.int64)
    r = np.concatenate([r, d])
    c = np.concatenate([c, d])
    v = np.concatenate([v, np.ones(n)])
    order = np.lexsort((r, c))          # CSC: by column, rows ascending
    r, c, v = r[order], c[order], v[order]
    col_ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(c, minlength=n), out=col_ptr[1:])
    return CscTriangle(n, col_ptr.astype(np.int32), r.astype(np.int32), v, substitution == 0)


def read_csc(path, substitution: int, seed: int = 0) -> CscTriangle:
    """The reference's -csc input (1-based pointers and rows); values 1..10. main.cu:247-294."""
    with open(path, "r") as f:
        tokens = np.array(f.read().split(), dtype=np.int64)
    if tokens.size < 3:
        raise ValueError(f"{path}: truncated")
    m, n, nnz = (int(t) for t in tokens[:3])
    if m != n:
        raise ValueError("the matrix is not square")
    if tokens.size < 3 + n + 1 + nnz:
        raise ValueError(f"{path}: truncated")
    col_ptr = tokens[3:3 + n + 1] - 1
    row_idx = tokens[3 + n + 1:3 + n + 1 + nnz] - 1
    rng = np.random.default_rng(seed)
    val = rng.integers(1, 11, size=nnz).astype(np.float64)
    return CscTriangle(n, col_ptr.astype(np.int32), row_idx.astype(np.int32), val, substitution == 0)


def manufactured_rhs(mat: CscTriangle, rhs: int = 1, seed: int = 0):
    """(x_ref, b) with x_ref entries 1..10 and b = L x_ref, row-major n x rhs. main.cu:333-358."""
    rng = np.random.default_rng(seed)
    x_ref = rng.integers(1, 11, size=(mat.n, rhs)).astype(np.float64)
    b = mat.matvec(x_ref)
    return x_ref, np.ascontiguousarray(b)

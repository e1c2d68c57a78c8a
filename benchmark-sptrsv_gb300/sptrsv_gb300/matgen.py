"""Seeded synthetic triangular systems in the reference's CSC layout.

The reference reads SuiteSparse matrices (SpTRSV_cuda/main.cu:142-319) and
replaces their values by ``rand()%10+1`` with a unit diagonal. This module
builds seeded synthetic systems with the shapes the benchmark workloads use,
in the same storage: 0-based ``int32`` column pointers and row indices, rows
sorted ascending inside each column, the diagonal first in a lower (forward)
column and last in an upper (backward) column (main.cu:221-231).

Values: off-diagonals ``U[-0.1, 0.1]``; diagonal
``U[1, 2] + sum|row off-diagonals| + sum|column off-diagonals|``, which makes
both the matrix and its transpose strictly diagonally dominant.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class CscTriangle:
    """A square triangular matrix in CSC form (reference main.cu:42-45)."""

    n: int
    col_ptr: np.ndarray  # int32 [n+1]
    row_idx: np.ndarray  # int32 [nnz]
    val: np.ndarray      # float64 [nnz]
    lower: bool          # True: forward substitution, False: backward

    @property
    def nnz(self) -> int:
        return int(self.row_idx.shape[0])

    @property
    def substitution(self) -> int:
        return 0 if self.lower else 1

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csc_matrix((self.val, self.row_idx, self.col_ptr), shape=(self.n, self.n))

    def transpose(self) -> "CscTriangle":
        """CSC of the transpose (the CSR of this matrix), rows kept sorted."""
        t = self.to_scipy().T.tocsc()
        t.sort_indices()
        return CscTriangle(self.n, t.indptr.astype(np.int32), t.indices.astype(np.int32),
                           t.data.astype(np.float64), not self.lower)

    def matvec(self, x: np.ndarray) -> np.ndarray:
        """b = L x for x of shape [n] or [n, rhs]."""
        return self.to_scipy() @ x


def _assemble_sorted(n: int, off_col: np.ndarray, off_row: np.ndarray, off_val: np.ndarray,
                     rng: np.random.Generator) -> CscTriangle:
    """Build lower CSC arrays from off-diagonals already grouped by column with rows
    ascending inside each column; the dominant diagonal goes first in every column."""
    a = np.abs(off_val)
    row_sum = np.bincount(off_row, weights=a, minlength=n)
    col_sum = np.bincount(off_col, weights=a, minlength=n)
    diag = rng.uniform(1.0, 2.0, size=n) + row_sum + col_sum
    per_col = np.bincount(off_col, minlength=n).astype(np.int64)
    col_ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(per_col + 1, out=col_ptr[1:])
    nnz = int(col_ptr[-1])
    row_idx = np.empty(nnz, dtype=np.int32)
    val = np.empty(nnz, dtype=np.float64)
    dpos = col_ptr[:-1]
    row_idx[dpos] = np.arange(n, dtype=np.int32)
    val[dpos] = diag
    if off_col.shape[0]:
        # the off-diagonals fill every slot after each column's diagonal, in order
        off = np.ones(nnz, dtype=bool)
        off[dpos] = False
        row_idx[off] = off_row
        val[off] = off_val
    return CscTriangle(n, col_ptr.astype(np.int32), row_idx, val, True)


def banded_random_lower(n: int, counts: np.ndarray, band: int, seed_or_rng, lower: bool = True
                        ) -> CscTriangle:
    """Lower triangle whose column j holds up to ``counts[j]`` distinct rows drawn
    uniformly from the open interval (j, min(j + band, n)); duplicates are dropped.
    ``lower=False`` returns the transpose (an upper triangle with the same values).

    The k draws of a column are produced already sorted, as order statistics of k
    uniforms (normalised partial sums of k+1 exponentials), so no global sort runs."""
    rng = seed_or_rng if isinstance(seed_or_rng, np.random.Generator) else np.random.default_rng(seed_or_rng)
    j = np.arange(n, dtype=np.int64)
    avail = np.maximum(np.minimum(j + band, n) - (j + 1), 0)
    k = np.minimum(np.asarray(counts, dtype=np.int64), avail)
    seg = k + 1
    seg_end = np.cumsum(seg) - 1                      # index of each column's closing exponential
    cs = np.cumsum(rng.standard_exponential(int(seg_end[-1]) + 1 if n else 0))
    base = np.zeros(n, dtype=np.float64)
    if n > 1:
        base[1:] = cs[seg_end[:-1]]
    total_w = cs[seg_end] - base if n else base
    col = np.repeat(j, k)
    draw = np.ones(cs.shape[0], dtype=bool)           # every partial sum but the closing ones
    draw[seg_end] = False
    u = (cs[draw] - np.repeat(base, k)) / np.repeat(total_w, k)
    span = np.repeat(avail, k)
    row = col + 1 + np.minimum((u * span).astype(np.int64), span - 1)
    if row.shape[0] > 1:
        keep = np.ones(row.shape[0], dtype=bool)
        keep[1:] = (row[1:] != row[:-1]) | (col[1:] != col[:-1])
        col, row = col[keep], row[keep]
    val = rng.uniform(-0.1, 0.1, size=col.shape[0])
    m = _assemble_sorted(n, col, row, val, rng)
    return m if lower else m.transpose()


def poisson_band(n: int, mean: float, band: int, seed: int, lower: bool = True) -> CscTriangle:
    """Poisson(mean) off-diagonals per column inside a band (the 10k-row and 1M-row systems)."""
    rng = np.random.default_rng(seed)
    counts = rng.poisson(mean, size=n)
    return banded_random_lower(n, counts, band, rng, lower)


def power_law_band(n: int, target_nnz: int, band: int, seed: int, alpha: float = 2.1,
                   kmax: int = 1000, lower: bool = True) -> CscTriangle:
    """Column off-diagonal counts drawn from P(k) ~ k^-alpha on [1, kmax], scaled by one
    common factor so that the total stored count (diagonal included) is close to
    ``target_nnz``, then capped at ``kmax``."""
    rng = np.random.default_rng(seed)
    ks = np.arange(1, kmax + 1, dtype=np.float64)
    pmf = ks ** (-alpha)
    cdf = np.cumsum(pmf / pmf.sum())
    raw = np.searchsorted(cdf, rng.random(n), side="right") + 1
    raw = np.minimum(raw, kmax)
    scale = (target_nnz - n) / float(raw.sum())
    for _ in range(4):   # account for the cap when matching the target count
        got = np.clip(np.rint(raw * scale), 1, kmax).sum()
        scale *= (target_nnz - n) / float(got)
    counts = np.clip(np.rint(raw * scale), 1, kmax).astype(np.int64)
    return banded_random_lower(n, counts, band, rng, lower)


def laplace2d_lower(grid: int, lower: bool = True) -> CscTriangle:
    """Lower triangle of the 5-point Laplacian on a grid x grid mesh in natural
    ordering: diagonal 4, off-diagonals -1. Unknown j = r*grid + c feeds j+1 (same
    mesh row) and j+grid (next mesh row); there are 2*grid-1 level sets."""
    n = grid * grid
    j = np.arange(n, dtype=np.int64)
    c = j % grid
    r = j // grid
    right = c < grid - 1
    down = r < grid - 1
    cnt = 1 + right.astype(np.int64) + down.astype(np.int64)
    col_ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(cnt, out=col_ptr[1:])
    nnz = int(col_ptr[-1])
    row_idx = np.empty(nnz, dtype=np.int64)
    val = np.empty(nnz, dtype=np.float64)
    start = col_ptr[:-1]
    row_idx[start] = j
    val[start] = 4.0
    p = start + 1
    row_idx[p[right]] = j[right] + 1
    val[p[right]] = -1.0
    q = start + 1 + right.astype(np.int64)
    row_idx[q[down]] = j[down] + grid
    val[q[down]] = -1.0
    m = CscTriangle(n, col_ptr.astype(np.int32), row_idx.astype(np.int32), val, True)
    return m if lower else m.transpose()


def random_small(n: int, density: float, seed: int, lower: bool = True) -> CscTriangle:
    """Dense-ish random triangle for small parity cases (any column may reach any later row)."""
    rng = np.random.default_rng(seed)
    counts = rng.binomial(np.maximum(n - 1 - np.arange(n), 0), density)
    return banded_random_lower(n, counts, n, rng, lower)


def chain(n: int, lower: bool = True) -> CscTriangle:
    """Bidiagonal chain: unknown j feeds j+1 only (n level sets)."""
    rng = np.random.default_rng(12345)
    counts = np.ones(n, dtype=np.int64)
    return banded_random_lower(n, counts, 2, rng, lower)


def diagonal(n: int, lower: bool = True) -> CscTriangle:
    """Diagonal matrix (one level set)."""
    rng = np.random.default_rng(777)
    return banded_random_lower(n, np.zeros(n, dtype=np.int64), 1, rng, lower)


def _explicit_lower(n: int, col: np.ndarray, row: np.ndarray, seed: int, lower: bool) -> CscTriangle:
    rng = np.random.default_rng(seed)
    val = rng.uniform(-0.1, 0.1, size=col.shape[0])
    m = _assemble_sorted(n, col.astype(np.int64), row.astype(np.int64), val, rng)
    return m if lower else m.transpose()


def dense_lower(n: int, seed: int = 5, lower: bool = True) -> CscTriangle:
    """Full lower triangle (every entry below the diagonal stored)."""
    col, row = np.tril_indices(n, -1)
    order = np.lexsort((col, row))   # group by column (row index of tril is the 2nd key)
    col, row = row[order], col[order]
    return _explicit_lower(n, col, row, seed, lower)


def star(n: int, lower: bool = True) -> CscTriangle:
    """Unknown 0 feeds every other row (one long column, n-1 independent rows)."""
    row = np.arange(1, n, dtype=np.int64)
    col = np.zeros(n - 1, dtype=np.int64)
    return _explicit_lower(n, col, row, 99, lower)


# ---------------------------------------------------------------- workloads

def system_10k(seed: int = 0) -> CscTriangle:
    """n=10,000, Poisson(8) off-diagonals per column within a band of 2000, seed 0."""
    return poisson_band(10_000, 8.0, 2000, seed)


def system_laplace_2m(lower: bool = True) -> CscTriangle:
    """5-point Laplacian lower triangle on 1414 x 1414 (n = 1,999,396, 2,827 levels)."""
    return laplace2d_lower(1414, lower)


POWER_LAW_N = 4_194_304


def system_powerlaw_4m(seed: int = 1, lower: bool = True, n: int = POWER_LAW_N,
                       target_nnz: int = 40_000_000, band: int = 50_000) -> CscTriangle:
    """n = 4,194,304, power-law column counts (alpha 2.1, cap 1000), ~40M stored entries,
    rows within j+1..j+50,000."""
    return power_law_band(n, target_nnz, band, seed, lower=lower)


def system_1m(seed: int = 2, lower: bool = True, n: int = 1_000_000) -> CscTriangle:
    """n = 1,000,000, Poisson(9) off-diagonals plus the diagonal, band 20,000."""
    return poisson_band(n, 9.0, 20_000, seed, lower)


def batch_uneven(count: int = 512, seed: int = 3, nmin: int = 1000, nmax: int = 200_000,
                 scale: float = 1.0) -> list[CscTriangle]:
    """Independent systems, even indices lower and odd upper; sizes log-uniform on
    [nmin, nmax] (times ``scale``), stored entries per column U{3..20} including the
    diagonal, band U[100, 10000] per system."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=count))
    sizes = np.maximum((sizes * scale).astype(np.int64), 2)
    out = []
    for s, n in enumerate(sizes):
        n = int(n)
        per_col = rng.integers(3, 21)          # average stored entries per column, incl. diagonal
        band = int(rng.integers(100, 10_001))
        counts = rng.poisson(per_col - 1, size=n)
        out.append(banded_random_lower(n, counts, band, rng, lower=(s % 2 == 0)))
    return out

"""Generates the Matrix Market fixtures in tests/golden/mtx/ and, for each, the
outputs of the reference's own input path, compiled from the reference
checkout by oracle/Makefile (`make -C oracle ref`):

  * the CSR that the reference's reader builds (SpTRSV_cuda/mmio_highlevel.h:8-134
    mmio_info and :137-296 mmio_data): rows in file order, symmetric and
    hermitian storage expanded, duplicates kept;
  * the unit-lower (forward) and unit-upper (backward) triangles that
    SpTRSV_cuda/main.cu:153-218 extracts from it: the entries strictly below
    (above) the diagonal of every CSR row plus an appended unit diagonal, then
    the reference's CSR -> CSC transposition (tranpose.h:6-43). Only the
    pattern is kept: the reference draws the triangle's values from rand().

The .mtx files are small synthetic matrices written by this script (seeded),
one per storage kind the reader distinguishes. Run from the repository root
with SPTRSV_REFERENCE_DIR set to the reference checkout:
    python tests/golden/make_mtx_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "benchmark-sptrsv_gb300"))

from oracle import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "mtx"


def _entries(n: int, per_row: float, seed: int, keep):
    """Seeded distinct (row, col) pairs, 0-based, in a shuffled order, filtered by keep(r, c)."""
    rng = np.random.default_rng(seed)
    cells = set()
    for r in range(n):
        for c in rng.choice(n, size=rng.poisson(per_row) + 1, replace=True):
            if keep(r, int(c)):
                cells.add((r, int(c)))
    cells = sorted(cells)
    order = rng.permutation(len(cells))
    return [cells[i] for i in order], rng


def write_mtx(path: Path, n: int, field: str, symmetry: str, entries, values, comments=()):
    lines = [f"%%MatrixMarket matrix coordinate {field} {symmetry}"]
    lines += [f"% {c}" for c in comments]
    lines.append(f"{n} {n} {len(entries)}")
    for (r, c), v in zip(entries, values):
        if field == "pattern":
            lines.append(f"{r + 1} {c + 1}")
        elif field == "integer":
            lines.append(f"{r + 1} {c + 1} {int(v)}")
        elif field == "complex":
            lines.append(f"{r + 1} {c + 1} {v[0]:.17g} {v[1]:.17g}")
        else:
            lines.append(f"{r + 1} {c + 1} {v:.17g}")
    path.write_text("\n".join(lines) + "\n")


def make_files() -> list[Path]:
    OUT.mkdir(exist_ok=True)
    files = []
    # general real: entries on both sides of the diagonal, some diagonals missing
    e, rng = _entries(9, 2.5, 1, lambda r, c: True)
    files.append(OUT / "general_real.mtx")
    write_mtx(files[-1], 9, "real", "general", e, rng.uniform(-5, 5, len(e)), ["seeded general matrix", "2 comments"])
    # symmetric real: lower storage (diagonal included)
    e, rng = _entries(12, 2.0, 2, lambda r, c: c <= r)
    files.append(OUT / "symmetric_real.mtx")
    write_mtx(files[-1], 12, "real", "symmetric", e, rng.uniform(-1, 1, len(e)))
    # pattern symmetric
    e, rng = _entries(15, 2.0, 3, lambda r, c: c <= r)
    files.append(OUT / "pattern_symmetric.mtx")
    write_mtx(files[-1], 15, "pattern", "symmetric", e, np.ones(len(e)))
    # integer general
    e, rng = _entries(10, 3.0, 4, lambda r, c: True)
    files.append(OUT / "integer_general.mtx")
    write_mtx(files[-1], 10, "integer", "general", e, rng.integers(-9, 10, len(e)))
    # skew-symmetric: strictly lower storage (the reference reads it as general)
    e, rng = _entries(8, 2.0, 5, lambda r, c: c < r)
    files.append(OUT / "skew_symmetric.mtx")
    write_mtx(files[-1], 8, "real", "skew-symmetric", e, rng.uniform(-1, 1, len(e)))
    # complex hermitian (the reader keeps the real part)
    e, rng = _entries(7, 2.0, 6, lambda r, c: c <= r)
    files.append(OUT / "complex_hermitian.mtx")
    write_mtx(files[-1], 7, "complex", "hermitian", e,
              list(zip(rng.uniform(-1, 1, len(e)), rng.uniform(-1, 1, len(e)))))
    return files


def extract_pattern(m: int, row_ptr, col_idx, substitution: int):
    """main.cu:153-218 on the reader's CSR: strict triangle of every row plus an
    appended unit diagonal, then the reference's transposition to CSC."""
    ptr = [0]
    idx = []
    for i in range(m):
        for j in range(row_ptr[i], row_ptr[i + 1]):
            c = int(col_idx[j])
            if (substitution == 0 and c < i) or (substitution == 1 and c > i):
                idx.append(c)
        idx.append(i)
        ptr.append(len(idx))
    ptr = np.array(ptr, dtype=np.int32)
    idx = np.array(idx, dtype=np.int32)
    imp = oracle.ref()
    cp, ri, _ = imp.transpose(ptr, idx, np.ones(idx.size), m)
    # main.cu:206-211 sorts the rows of every column (they come out ascending already)
    for c in range(m):
        ri[cp[c]:cp[c + 1]] = np.sort(ri[cp[c]:cp[c + 1]])
    return cp, ri


def main() -> int:
    if oracle.ref() is None:
        print("the reference build is required (set SPTRSV_REFERENCE_DIR and run make -C oracle ref)")
        return 1
    for f in make_files():
        m, n, rp, ci, v = oracle.ref_read_mtx(f)
        lp, li = extract_pattern(m, rp, ci, 0)
        up, ui = extract_pattern(m, rp, ci, 1)
        np.savez_compressed(f.with_suffix(".npz"), m=m, n=n, csr_ptr=rp, csr_idx=ci, csr_val=v,
                            lower_col_ptr=lp, lower_row_idx=li, upper_col_ptr=up, upper_row_idx=ui)
        print(f.name, m, n, rp[-1])
    return 0


if __name__ == "__main__":
    sys.exit(main())

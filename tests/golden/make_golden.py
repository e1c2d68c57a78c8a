"""Generates the golden fixtures in this directory by running the reference's
own serial code (SpTRSV_cuda/sptrsv_syncfree_serialref.h, tranpose.h,
findlevel.h), compiled from the reference checkout by oracle/Makefile
(`make -C oracle ref`), on small seeded systems.

Run from the repository root:  python tests/golden/make_golden.py
The fixtures are inputs plus the reference's outputs; the tests compare the
oracle port (oracle/sptrsv_oracle.c) and the CUDA library against them.
"""
from __future__ import annotations

import sys
import zlib
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "benchmark-sptrsv_gb300"))

from oracle import oracle  # noqa: E402
from sptrsv_gb300 import matgen  # noqa: E402

OUT = Path(__file__).resolve().parent


def hand4() -> matgen.CscTriangle:
    # L = [[1,0,0,0],[1,1,0,0],[0,2,1,0],[1,0,3,1]] in CSC, diagonal first.
    col_ptr = np.array([0, 3, 5, 7, 8], dtype=np.int32)
    row_idx = np.array([0, 1, 3, 1, 2, 2, 3, 3], dtype=np.int32)
    val = np.array([1, 1, 1, 1, 2, 1, 3, 1], dtype=np.float64)
    return matgen.CscTriangle(4, col_ptr, row_idx, val, True)


def unit_rand_values(m: matgen.CscTriangle, seed: int) -> matgen.CscTriangle:
    """The reference's test values: rand()%10+1 off the diagonal, unit diagonal (main.cu:168-186)."""
    rng = np.random.default_rng(seed)
    val = rng.integers(1, 11, size=m.nnz).astype(np.float64)
    diag_pos = m.col_ptr[:-1] if m.lower else m.col_ptr[1:] - 1
    val[diag_pos] = 1.0
    return matgen.CscTriangle(m.n, m.col_ptr, m.row_idx, val, m.lower)


def cases():
    yield "hand4_fwd", hand4(), 1, "ones_to_1234"
    yield "band2000_fwd", matgen.poisson_band(2000, 8.0, 400, seed=0), 1, "ones"
    yield "band2000_bwd", matgen.poisson_band(2000, 8.0, 400, seed=0, lower=False), 1, "ones"
    yield "laplace24_fwd", matgen.laplace2d_lower(24), 1, "ones"
    yield "laplace24_bwd", matgen.laplace2d_lower(24, lower=False), 1, "ones"
    yield "chain300_fwd", matgen.chain(300), 1, "normal"
    yield "diag100_bwd", matgen.diagonal(100, lower=False), 1, "normal"
    yield "dense64_fwd", matgen.dense_lower(64), 1, "normal"
    yield "star200_fwd", matgen.star(200), 1, "normal"
    yield "random500_rhs3_fwd", matgen.random_small(500, 0.02, seed=7), 3, "normal"
    yield "random500_rhs3_bwd", matgen.random_small(500, 0.02, seed=8, lower=False), 3, "normal"
    yield "unitrand_band1500_fwd", unit_rand_values(matgen.poisson_band(1500, 5.0, 300, seed=11), 11), 2, "randint"
    yield "unitrand_band1500_bwd", unit_rand_values(matgen.poisson_band(1500, 5.0, 300, seed=12, lower=False), 12), 1, "randint"
    yield "uneven3000_bwd", matgen.banded_random_lower(3000, np.random.default_rng(13).integers(2, 20, 3000), 500, 13,
                                                        lower=False), 4, "normal"


def main() -> int:
    ref = oracle.ref()
    if ref is None:
        print("reference build unavailable (needs the reference checkout)", file=sys.stderr)
        return 1
    for name, m, rhs, kind in cases():
        rng = np.random.default_rng(zlib.crc32(name.encode()))
        if kind == "ones_to_1234":
            x_true = np.array([1, 2, 3, 4], dtype=np.float64)
        elif kind == "ones":
            x_true = np.ones((m.n, rhs))
        elif kind == "randint":
            x_true = rng.integers(1, 11, size=(m.n, rhs)).astype(np.float64)
        else:
            x_true = rng.standard_normal((m.n, rhs))
        x_true = x_true.reshape(m.n, rhs)
        b = oracle.csc_spmv(m.col_ptr, m.row_idx, m.val, m.n, x_true)
        deg = ref.analyser(m.row_idx, m.n)
        x64 = ref.executor(m.col_ptr, m.row_idx, m.val, deg, m.n, m.substitution, rhs, b)
        x32 = ref.executor(m.col_ptr, m.row_idx, m.val.astype(np.float32), deg, m.n, m.substitution, rhs,
                           b.astype(np.float32))
        csr_ptr, csr_idx, csr_val = ref.transpose(m.col_ptr, m.row_idx, m.val, m.n)
        nl, lptr, litem = ref.findlevel(m.col_ptr, m.row_idx, m.n)
        stats = np.array(ref.findlevel_csc(m.col_ptr, m.row_idx, m.n), dtype=np.int32)
        np.savez_compressed(
            OUT / f"{name}.npz", n=np.int32(m.n), lower=np.int8(m.lower), rhs=np.int32(rhs),
            col_ptr=m.col_ptr, row_idx=m.row_idx, val=m.val, b=b.reshape(-1), x_true=x_true.reshape(-1),
            in_degree=deg, x64=x64, x32=x32, csr_ptr=csr_ptr, csr_idx=csr_idx, csr_val=csr_val,
            nlevel=np.int32(nl), level_ptr=lptr, level_item=litem, level_stats=stats)
        print(f"{name}: n={m.n} nnz={m.nnz} rhs={rhs} levels={nl} |x64-x_true|_1rel={oracle.l1_rel_err(x64, x_true):.2e}")
    return 0


if __name__ == "__main__":
    sys.exit(main())

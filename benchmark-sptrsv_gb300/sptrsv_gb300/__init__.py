"""sptrsv_gb300: sync-free sparse triangular solve on GB300 (sm_103a) behind a C ABI.

The compute path is libsptrsv_gb300.so (CUDA kernels for sm_103a). This package
is its Python binding: constants and status codes, the reference-compatible
host entry, the kernel-level analyser/executor surface, an analyse-once /
solve-many handle, seeded synthetic matrices, and the reference's input
preparation (Matrix Market / CSC files, triangle extraction, manufactured b).
"""
from . import matgen, mtx
from ._lib import (DTYPE_F32, DTYPE_F64, LAYOUT_COL_MAJOR, LAYOUT_ROW_MAJOR, OPT_WARP_AUTO, OPT_WARP_NNZ,
                   OPT_WARP_RHS, SCHED_AUTO, SCHED_LEVELSET, SCHED_PULL, SCHED_PUSH, SUBSTITUTION_BACKWARD,
                   SUBSTITUTION_FORWARD, SptrsvError, load)
from .solver import SyncFreeSolver, analyser, executor, sptrsv_syncfree_cuda


def sparse_triangular_solve(solver, values, b, recompute=False):
    """Differentiable x = op(L)^-1 b (see sptrsv_gb300.autograd)."""
    from .autograd import sparse_triangular_solve as _f
    return _f(solver, values, b, recompute)

__all__ = [
    "matgen", "mtx", "load", "sparse_triangular_solve", "SptrsvError", "SyncFreeSolver", "analyser", "executor", "sptrsv_syncfree_cuda",
    "SUBSTITUTION_FORWARD", "SUBSTITUTION_BACKWARD", "OPT_WARP_NNZ", "OPT_WARP_RHS", "OPT_WARP_AUTO",
    "LAYOUT_ROW_MAJOR", "LAYOUT_COL_MAJOR", "DTYPE_F64", "DTYPE_F32", "SCHED_AUTO", "SCHED_PUSH",
    "SCHED_PULL", "SCHED_LEVELSET",
]

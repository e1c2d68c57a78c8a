"""ctypes binding of libsptrsv_gb300.so (the C ABI declared in include/sptrsv_gb300.h).

The library is the only compute path: importing this module does not require a
GPU, but loading fails loudly when the shared library has not been built.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_ROOT / "_build" / "libsptrsv_gb300.so"
HEADER_PATH = PKG_ROOT.parent / "include" / "sptrsv_gb300.h"

# constants (include/sptrsv_gb300.h; values of SpTRSV_cuda/common.h:25-30)
SUBSTITUTION_FORWARD = 0
SUBSTITUTION_BACKWARD = 1
OPT_WARP_NNZ = 1
OPT_WARP_RHS = 2
OPT_WARP_AUTO = 3

OK = 0
ERR_NOT_SQUARE = -1
ERR_BAD_STRUCTURE = -2
ERR_INVALID = -3
ERR_CUDA = -4
ERR_TIMEOUT = -5
ERR_OOM = -6
ERR_STATE = -7
ERR_NOT_CONVERGED = -8
ERR_UNSUPPORTED = -9

LAYOUT_ROW_MAJOR = 0
LAYOUT_COL_MAJOR = 1
DTYPE_F64 = 0
DTYPE_F32 = 1

SCHED_AUTO = 0
SCHED_PUSH = 1
SCHED_PULL = 2
SCHED_LEVELSET = 3

OPTION_SCHEDULE = 0
OPTION_LANES = 1
OPTION_CHUNK = 2
OPTION_SMEM_TIER = 3
OPTION_EXACT = 4
OPTION_ORDER_BLOCK = 5
OPTION_TIMEOUT_MS = 6
OPTION_SYNC_CHECK = 7
OPTION_PROFILE = 8
OPTION_BLOCK = 9
OPTION_BACKOFF_NS = 10
OPTION_CTAS_PER_SM = 11
OPTION_STAGED = 12
OPTION_STAGE_ENTRIES = 13
OPTION_STAGES = 14
OPTION_FUSED_GRAD = 15
OPTION_WARP_SYNC = 16
OPTION_SPLIT = 17
OPTION_WSYNC_BATCH = 18
OPTION_IMPORT = 19
OPTION_UNIT_PIPELINE = 20
OPTION_FUSED_REFINE = 21
OPTION_OPT = 22
OPTION_RHS_TILE = 23
OPTION_STRETCH = 24

NOALLOC_MAX_N = 262144  # SPTRSV_NOALLOC_MAX_N


class SptrsvError(RuntimeError):
    """A non-zero sptrsv_status returned by the library."""

    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = status_string(status) if _LIB is not None else str(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


class Info(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int),
        ("nnz", ctypes.c_int),
        ("substitution", ctypes.c_int),
        ("nlevels", ctypes.c_int),
        ("parallelism_min", ctypes.c_int),
        ("parallelism_avg", ctypes.c_int),
        ("parallelism_max", ctypes.c_int),
        ("max_in_degree", ctypes.c_int),
        ("schedule", ctypes.c_int),
        ("lanes", ctypes.c_int),
        ("chunk", ctypes.c_int),
        ("order_block", ctypes.c_int),
        ("analysis_ms", ctypes.c_double),
        ("device_bytes", ctypes.c_size_t),
        ("block", ctypes.c_int),
        ("warp_sync", ctypes.c_int),
        ("staged", ctypes.c_int),
        ("split", ctypes.c_int),
        ("locality_permille", ctypes.c_int),
        ("unit_pipeline", ctypes.c_int),
        ("wsync_batch", ctypes.c_int),
        ("coarrive_permille", ctypes.c_int),
    ]


_VP = ctypes.c_void_p
_I = ctypes.c_int
_LL = ctypes.c_longlong
_D = ctypes.c_double
_PD = ctypes.POINTER(ctypes.c_double)

# name -> (restype, argtypes); the exported surface of include/sptrsv_gb300.h
SIGNATURES = {
    "sptrsv_gb300_status_string": (ctypes.c_char_p, [_I]),
    "sptrsv_gb300_version": (_I, []),
    "sptrsv_syncfree_cuda": (_I, [_VP, _VP, _VP, _I, _I, _I, _I, _I, _I, _VP, _VP, _VP, _VP]),
    "sptrsv_gb300_set_verbose": (None, [_I]),
    "sptrsv_gb300_set_bench_repeat": (None, [_I]),
    "sptrsv_gb300_syncfree_host": (_I, [_VP, _VP, _VP, _I, _I, _I, _I, _I, _I, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "sptrsv_gb300_analyser": (_I, [_VP, _I, _I, _VP, _VP]),
    "sptrsv_gb300_executor": (_I, [_VP, _VP, _VP, _VP, _VP, _I, _I, _I, _I, _VP, _VP, _VP]),
    "sptrsv_gb300_create": (_I, [ctypes.POINTER(_VP)]),
    "sptrsv_gb300_destroy": (_I, [_VP]),
    "sptrsv_gb300_set_option": (_I, [_VP, _I, _LL]),
    "sptrsv_gb300_get_option": (_I, [_VP, _I, ctypes.POINTER(_LL)]),
    "sptrsv_gb300_analyse": (_I, [_VP, _I, _I, _I, _VP, _VP, _I, _VP]),
    "sptrsv_gb300_get_info": (_I, [_VP, ctypes.POINTER(Info)]),
    "sptrsv_gb300_analyse_batch": (_I, [_VP, _I, _VP, _VP, _VP, _VP, _VP, _VP]),
    "sptrsv_gb300_batch_count": (_I, [_VP, ctypes.POINTER(_I)]),
    "sptrsv_gb300_levels": (_I, [_VP, _VP, _VP, _VP]),
    "sptrsv_gb300_csr": (_I, [_VP, _VP, _VP, _VP, _VP]),
    "sptrsv_gb300_set_values": (_I, [_VP, _VP, _I, _VP]),
    "sptrsv_gb300_solve": (_I, [_VP, _VP, _I, _I, _I, _VP, _VP, _VP]),
    "sptrsv_gb300_check": (_I, [_VP, _VP]),
    "sptrsv_gb300_solve_refine": (_I, [_VP, _VP, _I, _I, _VP, _VP, _D, _I, ctypes.POINTER(_I), _PD, _VP]),
    "sptrsv_gb300_solve_adjoint": (_I, [_VP, _VP, _I, _I, _I, _VP, _VP, _VP, _VP, _VP]),
    "sptrsv_gb300_grad_values": (_I, [_VP, _I, _I, _I, _VP, _VP, _VP, _VP]),
    "sptrsv_gb300_exec_ms": (_I, [_VP, _PD]),
    "sptrsv_gb300_graph_create": (_I, [_VP, _I, _I, _I, _I, _VP, _VP, _I, ctypes.POINTER(_VP), _VP]),
    "sptrsv_gb300_graph_launch": (_I, [_VP, _VP]),
    "sptrsv_gb300_graph_destroy": (_I, [_VP]),
    "sptrsv_gb300_tune": (_I, [_VP, _VP, _I, _I, _I, _VP, _VP, _I, _PD, _VP]),
    "sptrsv_gb300_solve_noalloc": (_I, [_VP, _VP, _VP, _I, _I, _I, _VP, _VP, _VP]),
}

_LIB: ctypes.CDLL | None = None


def load(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Load (once) and return the C-ABI library with typed signatures."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first (python benchmark-sptrsv_gb300/build.py "
            "or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def status_string(status: int) -> str:
    return load().sptrsv_gb300_status_string(int(status)).decode()


def check(status: int, what: str = "") -> None:
    if status != OK:
        raise SptrsvError(status, what)

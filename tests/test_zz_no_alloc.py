"""The allocation-free entry point (sptrsv_gb300_solve_noalloc) against the
handle solve, through the C ABI.

Some callers cannot allocate device memory themselves (a host framework that
owns the whole device-memory budget, or a latency-critical loop that cannot
take the synchronisation an allocation may imply); this entry point keeps its
scratch in a fixed array inside the library. Two calls in a row must both
match the allocating path to the tolerance the FP64 parity tests use (1e-12
relative, max norm): the second call shows the shared scratch is cleared
between calls. This file is collected last on purpose."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def relerr(x, ref):
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


def _p(t):
    return ctypes.c_void_p(int(t.data_ptr()))


@pytest.mark.parametrize("lower", [True, False])
def test_noalloc_matches_handle_solve_twice(cuda, built_lib, lower):
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.poisson_band(20_000, 8.0, 2000, seed=31, lower=lower)
    cp = cuda.from_numpy(m.col_ptr).cuda()
    ri = cuda.from_numpy(m.row_idx).cuda()
    va = cuda.from_numpy(m.val).cuda()
    ref_solver = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val)
    stream = ctypes.c_void_p(int(cuda.cuda.current_stream().cuda_stream))
    for call in range(2):
        b = cuda.from_numpy(np.random.default_rng(call).standard_normal(m.n)).cuda()
        ref = ref_solver.solve(b).cpu().numpy()
        x = cuda.full((m.n,), float("nan"), dtype=cuda.float64, device="cuda")
        rc = built_lib.sptrsv_gb300_solve_noalloc(_p(cp), _p(ri), _p(va), m.n, m.nnz, m.substitution, _p(b), _p(x),
                                                  stream)
        assert rc == 0, f"call {call}: status {rc}"
        assert relerr(x.cpu().numpy(), ref) <= TOL64, f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_array(cuda, built_lib):
    from sptrsv_gb300 import _lib
    n = _lib.NOALLOC_MAX_N + 1
    rc = built_lib.sptrsv_gb300_solve_noalloc(None, None, None, n, n, 0, None, None, None)
    assert rc == _lib.ERR_UNSUPPORTED

"""The allocation-free entry point (sptrsv_gb300_solve_noalloc), through the C ABI.

Some callers cannot allocate device memory themselves (a host framework that
owns the whole device-memory budget, or a latency-critical loop that cannot
take the synchronisation an allocation may imply); this entry point keeps its
scratch in a fixed array inside the library. Two calls in a row must both
match the FP64 oracle and the allocating path to the tolerance the FP64
parity tests use (1e-12 relative, max norm): the second call shows the shared
scratch is cleared between calls. Further cases: a system of exactly the
array's maximum size, malformed structure (a row index past n but inside the
array, so even a failed guard would stay in bounds), and an unchanged amount
of free device memory across a call. This file is collected last on purpose."""
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


def _stream(cuda):
    return ctypes.c_void_p(int(cuda.cuda.current_stream().cuda_stream))


def _device_arrays(cuda, m, row_idx=None):
    cp = cuda.from_numpy(m.col_ptr).cuda()
    ri = cuda.from_numpy(m.row_idx if row_idx is None else row_idx).cuda()
    va = cuda.from_numpy(m.val).cuda()
    return cp, ri, va


@pytest.mark.parametrize("lower", [True, False])
def test_noalloc_matches_oracle_and_handle_solve_twice(cuda, built_lib, oracle_port, lower):
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.poisson_band(20_000, 8.0, 2000, seed=31, lower=lower)
    cp, ri, va = _device_arrays(cuda, m)
    handle = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val)
    for call in range(2):
        b_h = np.random.default_rng(call).standard_normal(m.n)
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b_h)
        b = cuda.from_numpy(b_h).cuda()
        x = cuda.full((m.n,), float("nan"), dtype=cuda.float64, device="cuda")
        rc = built_lib.sptrsv_gb300_solve_noalloc(_p(cp), _p(ri), _p(va), m.n, m.nnz, m.substitution, _p(b), _p(x),
                                                  _stream(cuda))
        assert rc == 0, f"call {call}: status {rc}"
        x_h = x.cpu().numpy()
        assert relerr(x_h, ref) <= TOL64, f"call {call} vs the oracle"
        assert relerr(x_h, handle.solve(b).cpu().numpy()) <= TOL64, f"call {call} vs the handle solve"
    handle.close()


@pytest.mark.parametrize("lower", [True, False])
def test_noalloc_at_the_array_limit(cuda, built_lib, oracle_port, lower):
    """n == SPTRSV_NOALLOC_MAX_N: the last counter and partial-sum slots of the array are used."""
    from sptrsv_gb300 import _lib, matgen
    n = _lib.NOALLOC_MAX_N
    m = matgen.poisson_band(n, 4.0, 300, seed=37, lower=lower)
    assert m.n == n
    cp, ri, va = _device_arrays(cuda, m)
    b_h = np.random.default_rng(5).standard_normal(n)
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, n, m.substitution, b_h)
    b = cuda.from_numpy(b_h).cuda()
    for call in range(2):
        x = cuda.full((n,), float("nan"), dtype=cuda.float64, device="cuda")
        rc = built_lib.sptrsv_gb300_solve_noalloc(_p(cp), _p(ri), _p(va), n, m.nnz, m.substitution, _p(b), _p(x),
                                                  _stream(cuda))
        assert rc == 0, f"call {call}: status {rc}"
        assert relerr(x.cpu().numpy(), ref) <= TOL64, f"call {call}"


def test_noalloc_rejects_malformed_structure(cuda, built_lib, oracle_port):
    """A row index >= n (but below the array's size, so nothing could land outside the
    array even if the guard failed) returns BAD_STRUCTURE; so do decreasing column
    pointers. A correct call right after each one still solves."""
    from sptrsv_gb300 import _lib, matgen
    m = matgen.poisson_band(8000, 6.0, 500, seed=39, lower=True)
    assert m.n + 100 < _lib.NOALLOC_MAX_N
    b_h = np.random.default_rng(2).standard_normal(m.n)
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b_h)
    b = cuda.from_numpy(b_h).cuda()
    bad_row = m.row_idx.copy()
    col = 4321
    bad_row[m.col_ptr[col + 1] - 1] = m.n + 50
    bad_ptr = m.col_ptr.copy()
    bad_ptr[100] = bad_ptr[102]
    cases = [("row past n", m.col_ptr, bad_row), ("decreasing column pointers", bad_ptr, m.row_idx)]
    good_cp, good_ri, va = _device_arrays(cuda, m)
    for what, cp_h, ri_h in cases:
        cp = cuda.from_numpy(cp_h).cuda()
        ri = cuda.from_numpy(ri_h).cuda()
        x = cuda.zeros(m.n, dtype=cuda.float64, device="cuda")
        rc = built_lib.sptrsv_gb300_solve_noalloc(_p(cp), _p(ri), _p(va), m.n, m.nnz, 0, _p(b), _p(x), _stream(cuda))
        assert rc == _lib.ERR_BAD_STRUCTURE, f"{what}: status {rc}"
        rc = built_lib.sptrsv_gb300_solve_noalloc(_p(good_cp), _p(good_ri), _p(va), m.n, m.nnz, 0, _p(b), _p(x),
                                                  _stream(cuda))
        assert rc == 0, f"after {what}: status {rc}"
        assert relerr(x.cpu().numpy(), ref) <= TOL64, f"after {what}"


def test_noalloc_leaves_free_device_memory_unchanged(cuda, built_lib):
    """After a first (warm-up) call, another call changes the device's free memory by nothing."""
    from sptrsv_gb300 import matgen
    m = matgen.poisson_band(50_000, 8.0, 3000, seed=33, lower=False)
    cp, ri, va = _device_arrays(cuda, m)
    b = cuda.ones(m.n, dtype=cuda.float64, device="cuda")
    x = cuda.empty(m.n, dtype=cuda.float64, device="cuda")

    def call():
        rc = built_lib.sptrsv_gb300_solve_noalloc(_p(cp), _p(ri), _p(va), m.n, m.nnz, 1, _p(b), _p(x),
                                                  _stream(cuda))
        assert rc == 0

    call()
    cuda.cuda.synchronize()
    free0, _ = cuda.cuda.mem_get_info()
    for _ in range(3):
        call()
    cuda.cuda.synchronize()
    free1, _ = cuda.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_sizes_beyond_its_array(cuda, built_lib):
    from sptrsv_gb300 import _lib
    n = _lib.NOALLOC_MAX_N + 1
    rc = built_lib.sptrsv_gb300_solve_noalloc(None, None, None, n, n, 0, None, None, None)
    assert rc == _lib.ERR_UNSUPPORTED

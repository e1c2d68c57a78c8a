"""Error paths on the GPU: malformed structure is rejected on the host side of
the analysis, and a wait that can never finish returns SPTRSV_ERR_TIMEOUT
(bounded waits; nothing faults or hangs) and leaves the context usable."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solver(cuda, cp, ri, n, sub=0, **kw):
    from sptrsv_gb300 import SyncFreeSolver
    return SyncFreeSolver(np.asarray(cp, np.int32), np.asarray(ri, np.int32), n, sub, **kw)


def _status(fn):
    from sptrsv_gb300 import SptrsvError
    try:
        fn()
    except SptrsvError as e:
        return e.status
    return 0


@pytest.mark.parametrize("cp,ri,sub", [
    ([0, 1, 2, 3], [0, 2, 2], 0),           # column 1 misses its diagonal
    ([0, 2, 3, 4], [1, 0, 1, 2], 0),        # unsorted rows in column 0
    ([0, 1, 3, 4], [0, 0, 1, 2], 0),        # entry above the diagonal in a lower solve
    ([0, 2, 3, 4], [0, 1, 1, 2], 1),        # entry below the diagonal in an upper solve
    ([0, 1, 1, 3], [0, 1, 2], 0),           # empty column
    ([0, 2, 1, 3], [0, 1, 2], 0),           # decreasing column pointers
    ([0, 1, 2, 5], [0, 1, 2], 0),           # colPtr[n] != nnz
    ([0, 1, 2, 3], [0, 1, 7], 0),           # row out of range
])
def test_bad_structure_rejected(cuda, cp, ri, sub):
    from sptrsv_gb300 import _lib
    n = len(cp) - 1
    st = _status(lambda: _solver(cuda, cp, ri, n, sub))
    assert st == _lib.ERR_BAD_STRUCTURE


def test_zero_diagonal_rejected(cuda):
    from sptrsv_gb300 import _lib
    st = _status(lambda: _solver(cuda, [0, 2, 3], [0, 1, 1], 2, values=np.array([0.0, 1.0, 2.0])))
    assert st == _lib.ERR_BAD_STRUCTURE


def test_not_square(cuda, built_lib):
    import ctypes
    from sptrsv_gb300 import _lib
    h = ctypes.c_void_p()
    assert built_lib.sptrsv_gb300_create(ctypes.byref(h)) == 0
    assert built_lib.sptrsv_gb300_analyse(h, 3, 4, 4, None, None, 0, None) == _lib.ERR_NOT_SQUARE
    assert built_lib.sptrsv_gb300_solve(h, None, 0, 1, 0, None, None, None) == _lib.ERR_STATE
    assert built_lib.sptrsv_gb300_destroy(h) == 0


def test_undercounted_in_degree_times_out_then_recovers(cuda):
    """Kernel-level executor fed an in-degree one higher than the truth: the
    affected column can never become ready; the bounded wait reports a timeout."""
    from sptrsv_gb300 import _lib, analyser, executor, matgen, SptrsvError
    m = matgen.poisson_band(2000, 4.0, 100, seed=1)
    cp = cuda.from_numpy(m.col_ptr).cuda()
    ri = cuda.from_numpy(m.row_idx).cuda()
    va = cuda.from_numpy(m.val).cuda()
    b = cuda.ones(m.n, dtype=cuda.float64, device="cuda")
    deg = cuda.empty(m.n, dtype=cuda.int32, device="cuda")
    analyser(ri, m.n, m.nnz, deg)
    bad = deg.clone()
    bad[m.n // 2] += 1
    left = cuda.zeros(m.n, dtype=cuda.float64, device="cuda")
    x = cuda.zeros(m.n, dtype=cuda.float64, device="cuda")
    with pytest.raises(SptrsvError) as ei:
        executor(cp, ri, va, bad, left, m.n, 0, 1, 3, b, x)
    assert ei.value.status == _lib.ERR_TIMEOUT
    # the context is still usable and a correct call succeeds
    good = deg.clone()
    left.zero_()
    executor(cp, ri, va, good, left, m.n, 0, 1, 3, b, x)
    ref = m.to_scipy()
    r = ref @ x.cpu().numpy() - 1.0
    assert np.max(np.abs(r)) < 1e-12


def test_handle_timeout_option(cuda):
    """Timeouts are configurable per handle and validated."""
    from sptrsv_gb300 import _lib, matgen, SyncFreeSolver, SptrsvError
    m = matgen.poisson_band(500, 3.0, 50, seed=2)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, 0, values=m.val, timeout_ms=250)
    assert s.get_option(_lib.OPTION_TIMEOUT_MS) == 250
    with pytest.raises(SptrsvError):
        s.set_option(_lib.OPTION_TIMEOUT_MS, 0)


def test_split_option_validated(cuda):
    """Split lengths below 4 (other than 0 = off) are rejected; valid ones read back."""
    from sptrsv_gb300 import _lib, matgen, SyncFreeSolver, SptrsvError
    m = matgen.poisson_band(500, 3.0, 50, seed=2)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, 0, values=m.val)
    assert s.get_option(_lib.OPTION_SPLIT) == 32
    for bad in (-1, 1, 3):
        with pytest.raises(SptrsvError):
            s.set_option(_lib.OPTION_SPLIT, bad)
    for ok in (0, 4, 64):
        s.set_option(_lib.OPTION_SPLIT, ok)
        assert s.get_option(_lib.OPTION_SPLIT) == ok
    for bad in (-1, 3, 8):
        with pytest.raises(SptrsvError):
            s.set_option(_lib.OPTION_WSYNC_BATCH, bad)
    for ok in (0, 1, 2, 4):
        s.set_option(_lib.OPTION_WSYNC_BATCH, ok)
        assert s.get_option(_lib.OPTION_WSYNC_BATCH) == ok
    for bad in (-1, 2, 64, 100, 16384):
        with pytest.raises(SptrsvError):
            s.set_option(_lib.OPTION_UNIT_PIPELINE, bad)
    for ok in (0, 1, 128, 8192):
        s.set_option(_lib.OPTION_UNIT_PIPELINE, ok)
        assert s.get_option(_lib.OPTION_UNIT_PIPELINE) == ok


@pytest.mark.parametrize("cfg", [dict(schedule=2), dict(schedule=1),
                                 dict(schedule=2, staged=False, warp_sync=True, import_deps=True,
                                      order_block=64),
                                 dict(schedule=2, staged=False, warp_sync=True, unit_pipeline=1,
                                      order_block=64)])
def test_wait_budget_expires_cleanly_then_recovers(cuda, cfg):
    """Natural order on the 2-D Laplacian makes single waits last far longer than
    a 1 ms budget: the solve must come back with SPTRSV_ERR_TIMEOUT (every wait
    bounded, copies drained), and the same handle must solve correctly after the
    budget is raised."""
    from sptrsv_gb300 import SptrsvError, SyncFreeSolver, _lib, matgen
    m = matgen.laplace2d_lower(1000)
    b = cuda.from_numpy(m.matvec(np.ones(m.n))).cuda()
    kw = dict(order_block=1, chunk=64, timeout_ms=1)
    kw.update(cfg)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, **kw)
    with pytest.raises(SptrsvError) as ei:
        s.solve(b)
    assert ei.value.status == _lib.ERR_TIMEOUT
    s.set_option(_lib.OPTION_TIMEOUT_MS, 20_000)
    s.set_option(_lib.OPTION_ORDER_BLOCK, 10**9)
    s.set_values(m.val)
    x = s.solve(b)
    assert float((x - 1).abs().max()) < 1e-12


@pytest.mark.parametrize("fused", [1, 2])
def test_fused_refine_wait_budget_expires_cleanly_then_recovers(cuda, fused):
    """The fused refinement pass bounds its waits too: on a 200,000-long chain the
    CTAs that hold late chunks wait for every earlier chunk, far longer than a 1 ms
    budget, so the call reports SPTRSV_ERR_TIMEOUT; the handle then refines
    correctly with a larger budget."""
    from sptrsv_gb300 import SptrsvError, SyncFreeSolver, _lib, matgen
    m = matgen.chain(200_000)
    b = cuda.from_numpy(m.matvec(np.ones(m.n))).cuda()
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, schedule=2, order_block=1,
                       chunk=64, timeout_ms=1, fused_refine=fused)
    with pytest.raises(SptrsvError) as ei:
        s.solve_refine(b)
    assert ei.value.status == _lib.ERR_TIMEOUT
    s.set_option(_lib.OPTION_TIMEOUT_MS, 20_000)
    s.set_option(_lib.OPTION_ORDER_BLOCK, 10**9)
    s.set_values(m.val)
    x, it, est = s.solve_refine(b)
    assert float((x - 1).abs().max()) < 1e-10


def test_new_options_validate_and_round_trip(cuda):
    """SPTRSV_OPTION_OPT (1..3), SPTRSV_OPTION_RHS_TILE (0, 1, 2, 4),
    SPTRSV_OPTION_FUSED_REFINE (0..2) and SPTRSV_OPTION_STRETCH (boolean): valid
    values round-trip, others return SPTRSV_ERR_INVALID and leave the option as it was."""
    from sptrsv_gb300 import SptrsvError, SyncFreeSolver, _lib, matgen
    m = matgen.poisson_band(500, 4.0, 50, seed=1)
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val)
    cases = {_lib.OPTION_OPT: ([1, 2, 3], [0, 4, -1]), _lib.OPTION_RHS_TILE: ([0, 1, 2, 4], [3, 8, -1]),
             _lib.OPTION_FUSED_REFINE: ([0, 1, 2], [3, -1])}
    for opt, (good, bad) in cases.items():
        for v in good:
            s.set_option(opt, v)
            assert s.get_option(opt) == v
        for v in bad:
            with pytest.raises(SptrsvError) as ei:
                s.set_option(opt, v)
            assert ei.value.status == _lib.ERR_INVALID
            assert s.get_option(opt) == good[-1]
    for v in (0, 1):
        s.set_option(_lib.OPTION_STRETCH, v)
        assert s.get_option(_lib.OPTION_STRETCH) == v
    s.close()


def test_stretch_option_on_a_batch_changes_only_the_order(cuda, oracle_port):
    """A batch solved with and without the stretched level order (switching between
    them on one handle re-lays the schedule out) gives the same answers."""
    from sptrsv_gb300 import SyncFreeSolver, _lib, matgen
    systems = matgen.batch_uneven(count=24, seed=8, nmin=200, nmax=20_000)
    vals = np.concatenate([m.val for m in systems])
    bs = [np.random.default_rng(k).standard_normal((m.n, 2)) for k, m in enumerate(systems)]
    refs = [oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, bs[k])
            for k, m in enumerate(systems)]
    s = SyncFreeSolver(batch=[(m.col_ptr, m.row_idx, m.n, m.substitution) for m in systems], values=vals)
    b = cuda.from_numpy(np.concatenate(bs)).cuda()
    for stretch in (1, 0, 1):
        s.set_option(_lib.OPTION_STRETCH, stretch)
        s.set_values(vals)
        x = s.solve(b).cpu().numpy()
        for k in range(len(systems)):
            sl = slice(s.offsets[k], s.offsets[k + 1])
            assert np.max(np.abs(x[sl] - refs[k])) / np.max(np.abs(refs[k])) <= 1e-12, (stretch, k)
    s.close()

"""CUDA path vs the oracle, through the C ABI (ctypes binding).

Tolerances: the FP64 push executor accumulates with atomics in arbitrary
order, so it is checked to 1e-12 relative in the max norm against the FP64
oracle; the pull executor in exact mode repeats the serial executor's
operation order and must be bit-identical; FP32 solves are checked to 1e-5
relative against the FP64 oracle (and bit-identical to the FP32 oracle in
exact mode)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


def relerr(x, ref):
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    return float(np.max(np.abs(x - ref)) / max(np.max(np.abs(ref)), 1e-300))


def make_solver(cuda, g, **kw):
    from sptrsv_gb300 import SyncFreeSolver
    sub = 0 if int(g["lower"]) else 1
    return SyncFreeSolver(g["col_ptr"], g["row_idx"], int(g["n"]), sub, values=g["val"], **kw)


def b_tensor(cuda, g, dtype=np.float64):
    n, rhs = int(g["n"]), int(g["rhs"])
    return cuda.from_numpy(g["b"].reshape(n, rhs).astype(dtype)).cuda()


CONFIGS = [
    dict(schedule=1, lanes=1),
    dict(schedule=1, lanes=4),
    dict(schedule=1, lanes=32, order_block=1),
    dict(schedule=1, lanes=8, smem_tier=False, order_block=10**9),
    dict(schedule=2, lanes=1),
    dict(schedule=2, lanes=2, order_block=1),
    dict(schedule=2, lanes=8, order_block=10**9, chunk=64),
    dict(schedule=2, lanes=32, smem_tier=False),
    dict(schedule=2, staged=False, lanes=1),
    dict(schedule=2, staged=False, lanes=4, order_block=10**9),
    dict(schedule=2, chunk=32, stage_entries=64),
    dict(schedule=2, chunk=7, stage_entries=16, order_block=10**9, smem_tier=False),
    dict(schedule=2, chunk=4096, block=64, ctas_per_sm=1, backoff_ns=0),
    dict(schedule=2, chunk=100, stages=3, order_block=10**9),
    dict(schedule=2, chunk=33, stages=4, stage_entries=48, block=128),
    dict(schedule=2, staged=False, warp_sync=True),
    dict(schedule=2, staged=False, warp_sync=True, order_block=64, chunk=64, block=64),
    dict(schedule=2, staged=False, warp_sync=True, order_block=1, chunk=100, backoff_ns=0),
    dict(schedule=2, staged=False, warp_sync=True, split=0),
    dict(schedule=2, staged=False, warp_sync=True, split=4),
    dict(schedule=2, staged=False, warp_sync=True, split=5, chunk=32, smem_tier=False),
    dict(schedule=2, staged=False, warp_sync=True, split=4, order_block=64, chunk=96, block=64),
    dict(schedule=2, staged=False, warp_sync=True, wsync_batch=1),
    dict(schedule=2, staged=False, warp_sync=True, wsync_batch=2, order_block=64, chunk=64),
    dict(schedule=2, staged=False, warp_sync=True, wsync_batch=1, split=4),
    dict(schedule=2, staged=False, warp_sync=True, wsync_batch=2, split=5, chunk=32, smem_tier=False),
    dict(schedule=2, staged=False, warp_sync=True, order_block=64, chunk=64, block=64, import_deps=False),
    dict(schedule=2, staged=False, warp_sync=True, order_block=96, chunk=96, block=64, wsync_batch=1),
    dict(schedule=2, staged=False, warp_sync=True, order_block=200, chunk=200, block=128, wsync_batch=4),
    dict(schedule=2, staged=False, warp_sync=True, order_block=1000, chunk=1000, block=64, wsync_batch=1),
    dict(schedule=2, staged=False, warp_sync=True, order_block=777, chunk=777, block=64, wsync_batch=4),
    dict(schedule=3, lanes=1),
    dict(schedule=3, lanes=8),
]


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("cfg", CONFIGS, ids=lambda c: "-".join(f"{k}{v}" for k, v in c.items()))
def test_fp64_matches_oracle(cuda, name, cfg):
    g = load_golden(name)
    s = make_solver(cuda, g, **cfg)
    x = s.solve(b_tensor(cuda, g)).cpu().numpy()
    assert relerr(x, g["x64"]) <= TOL64
    # a second solve on the same handle (self-cleaning workspace) gives the same answer
    x2 = s.solve(b_tensor(cuda, g)).cpu().numpy()
    assert relerr(x2, g["x64"]) <= TOL64


PIPE_CONFIGS = [
    dict(order_block=1000, chunk=1000, unit_pipeline=1),
    dict(order_block=1000, chunk=1000, unit_pipeline=128, stage_entries=256, stages=2),
    dict(order_block=777, chunk=777, unit_pipeline=256, stage_entries=512, stages=4, wsync_batch=1),
    dict(order_block=300, chunk=300, unit_pipeline=128, stage_entries=128, wsync_batch=4),
    dict(order_block=64, chunk=64, unit_pipeline=1),
]


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("cfg", PIPE_CONFIGS, ids=lambda c: "-".join(f"{k}{v}" for k, v in c.items()))
def test_unit_pipeline_matches_oracle(cuda, name, cfg):
    """The unit pipeline (one consumer warp per order block, bulk-copy loader,
    ring of value slots) against the oracle, in FP64 and FP32; with small ring
    caps and stage buffers it wraps the ring, imports in-unit dependencies that
    lie too far back, and recycles every stage buffer many times."""
    g = load_golden(name)
    s = make_solver(cuda, g, schedule=2, staged=False, warp_sync=True, **cfg)
    x = s.solve(b_tensor(cuda, g)).cpu().numpy()
    assert relerr(x, g["x64"]) <= TOL64
    if int(g["rhs"]) == 1 and int(g["n"]) > cfg["order_block"]:
        assert s.info()["unit_pipeline"] == 1
    x2 = s.solve(b_tensor(cuda, g)).cpu().numpy()
    assert relerr(x2, g["x64"]) <= TOL64
    x32 = s.solve(b_tensor(cuda, g, np.float32)).cpu().numpy()
    assert relerr(x32, g["x64"]) <= TOL32


@pytest.mark.parametrize("ring,entries", [(128, 256), (1024, 2048), (1, 0)])
def test_unit_pipeline_mesh_and_band(cuda, oracle_port, ring, entries):
    """Larger blocked systems through the unit pipeline: a 2-D mesh in blocks of
    20 mesh rows and a random band whose in-unit dependencies often lie beyond
    the ring; FP64 results against the oracle."""
    from sptrsv_gb300 import SyncFreeSolver, matgen
    for m, ob in ((matgen.laplace2d_lower(100), 2000), (matgen.poisson_band(6000, 5.0, 400, seed=7), 1500),
                  (matgen.laplace2d_lower(100).transpose(), 2000)):
        rng = np.random.default_rng(11)
        bvec = rng.standard_normal(m.n)
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, bvec)
        s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, schedule=2, staged=False,
                           warp_sync=True, order_block=ob, chunk=ob, unit_pipeline=ring, stage_entries=entries)
        x = s.solve(cuda.from_numpy(bvec).cuda()).cpu().numpy()
        assert relerr(x, ref) <= TOL64
        assert s.info()["unit_pipeline"] == 1
        s.close()


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("order_block,staged,entries,wsync", [(1, True, 0, False), (256, True, 0, False),
                                                              (10**9, True, 0, False), (256, False, 0, False),
                                                              (10**9, True, 16, False), (256, False, 0, True)])
def test_exact_pull_is_bit_identical(cuda, name, order_block, staged, entries, wsync):
    g = load_golden(name)
    s = make_solver(cuda, g, schedule=2, exact=True, order_block=order_block, staged=staged,
                    stage_entries=entries, chunk=64 if entries else 0, warp_sync=wsync)
    x = s.solve(b_tensor(cuda, g)).cpu().numpy().ravel()
    assert np.array_equal(x.view(np.uint64), g["x64"].view(np.uint64))
    x32 = s.solve(b_tensor(cuda, g, np.float32)).cpu().numpy().ravel()
    assert np.array_equal(x32.view(np.uint32), g["x32"].view(np.uint32))


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("schedule", [1, 2, 3])
def test_fp32_close_to_fp64_oracle(cuda, name, schedule):
    g = load_golden(name)
    s = make_solver(cuda, g, schedule=schedule)
    x = s.solve(b_tensor(cuda, g, np.float32)).cpu().numpy()
    assert relerr(x, g["x64"]) <= TOL32


@pytest.mark.parametrize("schedule", [1, 2, 3])
def test_column_major_rhs(cuda, schedule):
    g = load_golden("uneven3000_bwd")
    n, rhs = int(g["n"]), int(g["rhs"])
    s = make_solver(cuda, g, schedule=schedule)
    b_rm = g["b"].reshape(n, rhs)
    b_cm = cuda.from_numpy(np.ascontiguousarray(b_rm.T)).cuda().t()   # [n, rhs] with stride (1, n)
    assert not b_cm.is_contiguous()
    x = s.solve(b_cm)
    assert x.stride() == (1, n)
    assert relerr(x.cpu().numpy(), g["x64"].reshape(n, rhs)) <= TOL64


@pytest.mark.parametrize("rhs", [31, 32, 40, 64])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_column_major_many_rhs_staged(cuda, oracle_port, rhs, dtype):
    """Column-major blocks of >= 32 right-hand sides go through row-major staging
    (transposes around the solve); results match the oracle, and in exact mode
    bit for bit."""
    from sptrsv_gb300 import SyncFreeSolver, matgen
    m = matgen.poisson_band(2500, 5.0, 250, seed=rhs, lower=(rhs % 2 == 1))
    B = np.random.default_rng(rhs).standard_normal((m.n, rhs))
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, exact=True)
    if dtype == "f64":
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, B)
        b_cm = cuda.from_numpy(np.ascontiguousarray(B.T)).cuda().t()
        x = s.solve(b_cm)
        assert x.stride() == (1, m.n)
        xe = x.cpu().numpy()
        assert np.array_equal(xe.view(np.uint64), ref.view(np.uint64))
    else:
        ref32 = oracle_port.solve(m.col_ptr, m.row_idx, m.val.astype(np.float32), m.n, m.substitution,
                                  B.astype(np.float32))
        b_cm = cuda.from_numpy(np.ascontiguousarray(B.T.astype(np.float32))).cuda().t()
        x = s.solve(b_cm, values=cuda.from_numpy(m.val.astype(np.float32)).cuda())
        assert x.stride() == (1, m.n)
        assert np.array_equal(x.cpu().numpy().view(np.uint32), ref32.view(np.uint32))


@pytest.mark.parametrize("rhs", [1, 3, 5, 16, 33, 64, 70])
@pytest.mark.parametrize("schedule,wsync,ob", [(1, False, None), (2, False, None), (3, False, None),
                                               (2, True, None), (2, True, 128)])
def test_many_rhs_against_oracle(cuda, oracle_port, rhs, schedule, wsync, ob):
    from sptrsv_gb300 import matgen
    m = matgen.poisson_band(3000, 6.0, 300, seed=rhs, lower=(rhs % 2 == 0))
    b = np.random.default_rng(rhs).standard_normal((m.n, rhs))
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
    from sptrsv_gb300 import SyncFreeSolver
    kw = dict(order_block=ob, chunk=ob) if ob else {}
    s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, schedule=schedule,
                       warp_sync=wsync, staged=not wsync, **kw)
    x = s.solve(cuda.from_numpy(b).cuda()).cpu().numpy()
    assert relerr(x, ref) <= TOL64
    s.set_option(4, 1)  # exact
    if schedule == 2:
        xe = s.solve(cuda.from_numpy(b).cuda()).cpu().numpy()
        assert np.array_equal(xe.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("name", golden_names())
def test_analysis_products_match_reference(cuda, name):
    g = load_golden(name)
    s = make_solver(cuda, g)
    info = s.info()
    assert info["nlevels"] == int(g["nlevel"])
    nl, pmin, pavg, pmax = (int(v) for v in g["level_stats"])
    assert (info["parallelism_min"], info["parallelism_avg"], info["parallelism_max"]) == (pmin, pavg, pmax)
    lp, li = s.levels()
    lp, li = lp.cpu().numpy(), li.cpu().numpy()
    np.testing.assert_array_equal(lp, g["level_ptr"])
    for lv in range(nl):   # same rows per level (the reference lists them in discovery order)
        a, b = lp[lv], lp[lv + 1]
        np.testing.assert_array_equal(np.sort(li[a:b]), np.sort(g["level_item"][a:b]))
    rp, ci, src = (t.cpu().numpy() for t in s.csr())
    np.testing.assert_array_equal(rp, g["csr_ptr"])
    np.testing.assert_array_equal(ci, g["csr_idx"])
    np.testing.assert_array_equal(g["val"][src], g["csr_val"])


@pytest.mark.parametrize("name", golden_names())
def test_kernel_level_surface(cuda, name):
    from sptrsv_gb300 import analyser, executor
    g = load_golden(name)
    n, rhs = int(g["n"]), int(g["rhs"])
    sub = 0 if int(g["lower"]) else 1
    cp = cuda.from_numpy(g["col_ptr"]).cuda()
    ri = cuda.from_numpy(g["row_idx"]).cuda()
    va = cuda.from_numpy(g["val"]).cuda()
    deg = cuda.empty(n, dtype=cuda.int32, device="cuda")
    analyser(ri, n, ri.numel(), deg)
    np.testing.assert_array_equal(deg.cpu().numpy(), g["in_degree"])
    for opt in (1, 2, 3):
        d2 = deg.clone()
        left = cuda.zeros(n * rhs, dtype=cuda.float64, device="cuda")
        x = cuda.zeros(n * rhs, dtype=cuda.float64, device="cuda")
        executor(cp, ri, va, d2, left, n, sub, rhs, opt, cuda.from_numpy(g["b"]).cuda(), x)
        assert relerr(x.cpu().numpy(), g["x64"]) <= TOL64


@pytest.mark.parametrize("name", ["hand4_fwd", "unitrand_band1500_fwd", "unitrand_band1500_bwd", "random500_rhs3_bwd"])
def test_reference_compatible_host_entry(cuda, name):
    from sptrsv_gb300 import sptrsv_syncfree_cuda
    g = load_golden(name)
    n, rhs = int(g["n"]), int(g["rhs"])
    sub = 0 if int(g["lower"]) else 1
    x = np.zeros(n * rhs)
    r = sptrsv_syncfree_cuda(g["col_ptr"], g["row_idx"], g["val"], n, n, g["row_idx"].size, sub, rhs, 3, x, g["b"],
                             g["x_true"], repeat=3)
    assert r["status"] == 0
    assert r["l1_err"] < 1e-4           # the reference's own acceptance test
    assert relerr(x, g["x64"]) <= TOL64
    assert r["gflops"] > 0
    r = sptrsv_syncfree_cuda(g["col_ptr"], g["row_idx"], g["val"], n, n + 1, g["row_idx"].size, sub, rhs, 3, x,
                             g["b"], None, repeat=1)
    assert r["status"] == -1


def test_full_size_properties_laplace(cuda, oracle_port):
    """The 2M-row Laplacian at full size: every schedule agrees with the oracle."""
    from sptrsv_gb300 import SyncFreeSolver, matgen
    for lower in (True, False):
        m = matgen.system_laplace_2m(lower=lower)
        x_true = np.ones(m.n)
        b = m.matvec(x_true)
        ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)
        for sched in (1, 2):
            s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, schedule=sched)
            x = s.solve(cuda.from_numpy(b).cuda()).cpu().numpy()
            assert relerr(x, ref) <= TOL64
            assert relerr(x, x_true) <= 1e-10
            s.close()
        s = SyncFreeSolver(m.col_ptr, m.row_idx, m.n, m.substitution, values=m.val, schedule=2, exact=True)
        x = s.solve(cuda.from_numpy(b).cuda()).cpu().numpy()
        assert np.array_equal(x.view(np.uint64), ref.view(np.uint64))
        assert s.info()["nlevels"] == 2 * 1414 - 1


def test_kernel_level_executor_two_threads_two_streams(cuda, oracle_port):
    """Two host threads, each on its own stream, run the kernel-level analyser and
    executor at the same time on different systems: the library keeps one control
    block (ticket, done and error words) per stream, so neither call disturbs the other."""
    import threading

    from sptrsv_gb300 import analyser, executor, matgen
    systems = [matgen.poisson_band(30_000, 6.0, 3000, seed=41, lower=True),
               matgen.poisson_band(24_000, 9.0, 1500, seed=42, lower=False)]
    refs, outs, errors = [], [None, None], []
    for k, m in enumerate(systems):
        b = np.random.default_rng(k).standard_normal(m.n)
        refs.append((b, oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, b)))

    def run(k):
        try:
            m = systems[k]
            stream = cuda.cuda.Stream()
            with cuda.cuda.stream(stream):
                cp = cuda.from_numpy(m.col_ptr).cuda()
                ri = cuda.from_numpy(m.row_idx).cuda()
                va = cuda.from_numpy(m.val).cuda()
                b = cuda.from_numpy(refs[k][0]).cuda()
                deg0 = cuda.empty(m.n, dtype=cuda.int32, device="cuda")
                analyser(ri, m.n, m.nnz, deg0, stream=stream)
                res = []
                for _ in range(6):
                    deg = deg0.clone()
                    left = cuda.zeros(m.n, dtype=cuda.float64, device="cuda")
                    x = cuda.zeros(m.n, dtype=cuda.float64, device="cuda")
                    executor(cp, ri, va, deg, left, m.n, m.substitution, 1, 3, b, x, stream=stream)
                    res.append(x.cpu().numpy())
                outs[k] = res
        except Exception as exc:  # noqa: BLE001 - reported by the main thread
            errors.append(exc)

    threads = [threading.Thread(target=run, args=(k,)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for k in range(2):
        for x in outs[k]:
            assert relerr(x, refs[k][1]) <= TOL64


def test_kernel_level_executor_rejects_row_out_of_range(cuda, oracle_port):
    """A row index >= m makes the kernel-level executor return BAD_STRUCTURE without
    writing through it. The counters and partial sums are allocated twice as long, so
    the planted row stays inside them even if the guard failed; their tails must stay
    untouched."""
    from sptrsv_gb300 import _lib, analyser, matgen
    m = matgen.poisson_band(5000, 5.0, 400, seed=43, lower=True)
    row_idx = m.row_idx.copy()
    col = 1000
    row_idx[m.col_ptr[col + 1] - 1] = m.n + 7     # last (largest) row of the column
    cp = cuda.from_numpy(m.col_ptr).cuda()
    ri = cuda.from_numpy(row_idx).cuda()
    va = cuda.from_numpy(m.val).cuda()
    deg = cuda.zeros(2 * m.n, dtype=cuda.int32, device="cuda")
    analyser(cuda.from_numpy(m.row_idx).cuda(), m.n, m.nnz, deg)
    left = cuda.zeros(2 * m.n, dtype=cuda.float64, device="cuda")
    b = cuda.ones(m.n, dtype=cuda.float64, device="cuda")
    x = cuda.zeros(m.n, dtype=cuda.float64, device="cuda")
    import ctypes
    stream = ctypes.c_void_p(int(cuda.cuda.current_stream().cuda_stream))
    p = lambda t: ctypes.c_void_p(int(t.data_ptr()))  # noqa: E731
    rc = _lib.load().sptrsv_gb300_executor(p(cp), p(ri), p(va), p(deg), p(left), m.n, 0, 1, 3, p(b), p(x), stream)
    assert rc == _lib.ERR_BAD_STRUCTURE
    assert int(deg[m.n:].abs().sum()) == 0
    assert float(left[m.n:].abs().sum()) == 0.0
    # the per-stream control block is usable again after the error
    deg2 = cuda.empty(m.n, dtype=cuda.int32, device="cuda")
    analyser(cuda.from_numpy(m.row_idx).cuda(), m.n, m.nnz, deg2)
    left2 = cuda.zeros(m.n, dtype=cuda.float64, device="cuda")
    rc = _lib.load().sptrsv_gb300_executor(p(cp), p(cuda.from_numpy(m.row_idx).cuda()), p(va), p(deg2), p(left2),
                                           m.n, 0, 1, 3, p(b), p(x), stream)
    assert rc == 0
    ref = oracle_port.solve(m.col_ptr, m.row_idx, m.val, m.n, m.substitution, np.ones(m.n))
    assert relerr(x.cpu().numpy(), ref) <= TOL64

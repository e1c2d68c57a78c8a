"""Host-side mirror of the reference's solver interface over the C ABI.

``sptrsv_syncfree_cuda`` keeps the reference signature and meaning
(SpTRSV_cuda/sptrsv_syncfree_cuda.h:409-421) on NumPy host arrays;
``analyser`` / ``executor`` mirror its two kernels (:8-19, :21-107/:290-407)
on device tensors; ``SyncFreeSolver`` is the analyse-once / solve-many handle.
PyTorch only supplies device memory and the current stream.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import (DTYPE_F32, DTYPE_F64, LAYOUT_COL_MAJOR, LAYOUT_ROW_MAJOR, SCHED_AUTO, SptrsvError, check,
                   load)


def _torch():
    import torch
    return torch


def _ptr(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if t is None else int(t.data_ptr()))


def _stream_ptr(stream=None) -> ctypes.c_void_p:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(int(s.cuda_stream))


def _np_ptr(a) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if a is None else a.ctypes.data)


# ------------------------------------------------------------------ reference host surface
def sptrsv_syncfree_cuda(col_ptr, row_idx, val, m, n, nnz, substitution, rhs, opt, x, b, x_ref=None,
                         repeat: int | None = None, verbose: bool = False):
    """Reference-compatible host entry (sptrsv_syncfree_cuda.h:409-421) on NumPy arrays.

    ``x`` (float64, n*rhs, row-major) is written in place. Returns a dict with the
    status (0, or -1 for a non-square matrix like the reference), GFLOPS of the
    average solve, solve/analysis milliseconds and the L1-relative error vs x_ref.
    """
    lib = load()
    col_ptr = np.ascontiguousarray(col_ptr, dtype=np.int32)
    row_idx = np.ascontiguousarray(row_idx, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    if x_ref is not None:
        x_ref = np.ascontiguousarray(x_ref, dtype=np.float64)
    if not (x.flags["C_CONTIGUOUS"] and x.dtype == np.float64):
        raise ValueError("x must be a C-contiguous float64 array")
    if repeat is not None:
        lib.sptrsv_gb300_set_bench_repeat(int(repeat))
    lib.sptrsv_gb300_set_verbose(1 if verbose else 0)
    gflops = ctypes.c_double(0.0)
    solve_ms = ctypes.c_double(0.0)
    an_ms = ctypes.c_double(0.0)
    err = ctypes.c_double(float("nan"))
    st = lib.sptrsv_gb300_syncfree_host(_np_ptr(col_ptr), _np_ptr(row_idx), _np_ptr(val), int(m), int(n),
                                        int(nnz), int(substitution), int(rhs), int(opt), _np_ptr(x), _np_ptr(b),
                                        _np_ptr(x_ref), ctypes.byref(gflops), ctypes.byref(solve_ms),
                                        ctypes.byref(an_ms), ctypes.byref(err))
    if repeat is not None:
        lib.sptrsv_gb300_set_bench_repeat(100)
    return {"status": st, "gflops": gflops.value, "solve_ms": solve_ms.value, "analysis_ms": an_ms.value,
            "l1_err": err.value}


# ------------------------------------------------------------------ reference kernel surface
def analyser(row_idx, m: int, nnz: int, in_degree, stream=None) -> None:
    """in_degree[r] = stored entries of row r, diagonal included (sptrsv_syncfree_cuda.h:8-19)."""
    check(load().sptrsv_gb300_analyser(_ptr(row_idx), int(m), int(nnz), _ptr(in_degree), _stream_ptr(stream)),
          "analyser")


def executor(col_ptr, row_idx, val, in_degree, left_sum, m: int, substitution: int, rhs: int, opt: int, b, x,
             stream=None) -> None:
    """Warp-per-column push executor on caller-owned counters (sptrsv_syncfree_cuda.h:21-107, :290-407).
    in_degree is consumed (counts down to 1) and left_sum accumulates, as in the reference."""
    check(load().sptrsv_gb300_executor(_ptr(col_ptr), _ptr(row_idx), _ptr(val), _ptr(in_degree), _ptr(left_sum),
                                       int(m), int(substitution), int(rhs), int(opt), _ptr(b), _ptr(x),
                                       _stream_ptr(stream)), "executor")


# ------------------------------------------------------------------ handle API
class SyncFreeSolver:
    """Analyse once, solve many: a handle of libsptrsv_gb300 bound to torch CUDA tensors.

    Keyword options map one to one onto ``SPTRSV_OPTION_*``; an option left at
    None keeps the library default, which with the automatic schedule is the
    plan chosen from the analysis (``info()`` reports the settings in effect).
    ``batch=[(col_ptr, row_idx, n, substitution), ...]`` analyses independent
    systems as one block-diagonal index space solved in one launch."""

    def __init__(self, col_ptr=None, row_idx=None, n: int | None = None, substitution: int = 0, *, values=None,
                 batch=None,
                 schedule: int | None = None, lanes: int | None = None, chunk: int | None = None,
                 order_block: int | None = None, exact: bool | None = None, smem_tier: bool | None = None,
                 timeout_ms: int | None = None, sync_check: bool | None = None, profile: bool | None = None,
                 block: int | None = None, backoff_ns: int | None = None, ctas_per_sm: int | None = None,
                 staged: bool | None = None, stage_entries: int | None = None, stages: int | None = None,
                 warp_sync: bool | None = None, split: int | None = None, wsync_batch: int | None = None,
                 import_deps: bool | None = None, unit_pipeline: int | None = None, fused_grad: bool | None = None,
                 fused_refine: int | None = None, opt: int | None = None, rhs_tile: int | None = None,
                 stretch: bool | None = None, stream=None):
        torch = _torch()
        self._lib = load()
        self.device = torch.device("cuda", torch.cuda.current_device())
        self.batch = None
        if batch is not None:
            # independent triangles [(col_ptr, row_idx, n, substitution), ...] solved together
            cps, ris, ns, nnzs, subs = [], [], [], [], []
            for cp, ri, nn, sub in batch:
                cp = np.asarray(cp, dtype=np.int32)
                ri = np.asarray(ri, dtype=np.int32)
                cps.append(cp)
                ris.append(ri)
                ns.append(int(nn))
                nnzs.append(int(ri.size))
                subs.append(int(sub))
            self.batch = (np.array(ns, dtype=np.int32), np.array(nnzs, dtype=np.int32), np.array(subs, dtype=np.int32))
            self.col_ptr = self._as_dev(np.concatenate(cps), torch.int32)
            self.row_idx = self._as_dev(np.concatenate(ris) if ris else np.zeros(0, np.int32), torch.int32)
            self.n = int(sum(ns))
            self.nnz = int(sum(nnzs))
            self.substitution = subs[0] if subs else 0
            self.offsets = np.concatenate([[0], np.cumsum(ns)]).astype(np.int64)
        else:
            self.col_ptr = self._as_dev(col_ptr, torch.int32)
            self.row_idx = self._as_dev(row_idx, torch.int32)
            self.n = int(self.col_ptr.numel() - 1) if n is None else int(n)
            self.nnz = int(self.row_idx.numel())
            self.substitution = int(substitution)
        h = ctypes.c_void_p()
        check(self._lib.sptrsv_gb300_create(ctypes.byref(h)), "create")
        self._h = h
        # only the options given here are set; the rest keep the library's
        # defaults (with the automatic schedule, the plan chosen at analysis)
        for opt, v in ((_lib.OPTION_SCHEDULE, schedule), (_lib.OPTION_LANES, lanes), (_lib.OPTION_CHUNK, chunk),
                       (_lib.OPTION_ORDER_BLOCK, order_block), (_lib.OPTION_EXACT, exact),
                       (_lib.OPTION_SMEM_TIER, smem_tier), (_lib.OPTION_TIMEOUT_MS, timeout_ms),
                       (_lib.OPTION_SYNC_CHECK, sync_check), (_lib.OPTION_PROFILE, profile),
                       (_lib.OPTION_BLOCK, block), (_lib.OPTION_BACKOFF_NS, backoff_ns),
                       (_lib.OPTION_CTAS_PER_SM, ctas_per_sm), (_lib.OPTION_STAGED, staged),
                       (_lib.OPTION_STAGE_ENTRIES, stage_entries), (_lib.OPTION_STAGES, stages),
                       (_lib.OPTION_WARP_SYNC, warp_sync), (_lib.OPTION_SPLIT, split),
                       (_lib.OPTION_WSYNC_BATCH, wsync_batch), (_lib.OPTION_IMPORT, import_deps),
                       (_lib.OPTION_UNIT_PIPELINE, unit_pipeline),
                       (_lib.OPTION_FUSED_GRAD, fused_grad), (_lib.OPTION_FUSED_REFINE, fused_refine),
                       (_lib.OPTION_OPT, opt), (_lib.OPTION_RHS_TILE, rhs_tile),
                       (_lib.OPTION_STRETCH, stretch)):
            if v is not None:
                self.set_option(opt, int(v))
        self._stream = stream
        self.analyse()
        self.values = None
        if values is not None:
            self.set_values(values)

    def _as_dev(self, a, dtype):
        torch = _torch()
        if isinstance(a, np.ndarray):
            a = torch.from_numpy(np.ascontiguousarray(a))
        return a.to(device=self.device, dtype=dtype).contiguous()

    def set_option(self, option: int, value: int) -> None:
        check(self._lib.sptrsv_gb300_set_option(self._h, int(option), int(value)), f"set_option({option})")

    def get_option(self, option: int) -> int:
        v = ctypes.c_longlong(0)
        check(self._lib.sptrsv_gb300_get_option(self._h, int(option), ctypes.byref(v)), "get_option")
        return int(v.value)

    def analyse(self) -> None:
        if self.batch is not None:
            ns, nnzs, subs = self.batch
            check(self._lib.sptrsv_gb300_analyse_batch(self._h, int(ns.size), _np_ptr(ns), _np_ptr(nnzs),
                                                       _np_ptr(subs), _ptr(self.col_ptr), _ptr(self.row_idx),
                                                       _stream_ptr(self._stream)), "analyse_batch")
            return
        check(self._lib.sptrsv_gb300_analyse(self._h, self.n, self.n, self.nnz, _ptr(self.col_ptr),
                                             _ptr(self.row_idx), self.substitution, _stream_ptr(self._stream)),
              "analyse")

    def set_values(self, values) -> None:
        torch = _torch()
        v = values if isinstance(values, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(values))
        v = v.to(self.device).contiguous()
        if v.dtype not in (torch.float64, torch.float32):
            v = v.to(torch.float64)
        dt = DTYPE_F64 if v.dtype == torch.float64 else DTYPE_F32
        check(self._lib.sptrsv_gb300_set_values(self._h, _ptr(v), dt, _stream_ptr(self._stream)), "set_values")
        self.values = v

    def solve(self, b, values=None, *, out=None):
        """Solve op(L) X = B. ``b``: [n] or [n, rhs] float64/float32 CUDA tensor; a column-major
        [n, rhs] view (stride (1, n)) is solved in place of layout without a copy. Returns x with
        b's layout and dtype."""
        torch = _torch()
        if b.dim() == 1:
            b2 = b.reshape(-1, 1)
        else:
            b2 = b
        if b2.shape[0] != self.n:
            raise ValueError(f"b has {b2.shape[0]} rows, the matrix has {self.n}")
        rhs = int(b2.shape[1])
        if b2.is_contiguous():
            layout = LAYOUT_ROW_MAJOR
        elif b2.t().is_contiguous():
            layout = LAYOUT_COL_MAJOR
        else:
            b2 = b2.contiguous()
            layout = LAYOUT_ROW_MAJOR
        if b2.dtype == torch.float64:
            dt = DTYPE_F64
        elif b2.dtype == torch.float32:
            dt = DTYPE_F32
        else:
            raise TypeError("b must be float64 or float32")
        if out is None:
            if layout == LAYOUT_ROW_MAJOR:
                out = torch.empty_like(b2, memory_format=torch.contiguous_format)
            else:
                out = torch.empty((rhs, self.n), dtype=b2.dtype, device=b2.device).t()
        vptr = ctypes.c_void_p(0)
        if values is not None:
            v = values.to(self.device).contiguous()
            self.values = v
            vptr = _ptr(v)
        st = self._lib.sptrsv_gb300_solve(self._h, vptr, dt, rhs, layout, _ptr(b2), _ptr(out),
                                          _stream_ptr(self._stream))
        check(st, "solve")
        return out.reshape(b.shape) if b.dim() == 1 else out

    def solve_refine(self, b, values=None, *, tol: float = 1e-12, max_iter: int = 10, out=None):
        """FP32 storage/solve + FP64-residual iterative refinement (b float64). Returns
        (x, iterations, estimated relative forward error). With the default
        ``fused_refine`` the first FP32 solve, FP64 residual and FP32 correction run
        as one pass over the dependency DAG."""
        torch = _torch()
        b2, layout = self._layout_of(b)
        if b2.dtype != torch.float64:
            raise TypeError("solve_refine takes float64 right-hand sides")
        rhs = int(b2.shape[1])
        if out is None:
            out = (torch.empty_like(b2, memory_format=torch.contiguous_format) if layout == LAYOUT_ROW_MAJOR
                   else torch.empty((rhs, self.n), dtype=b2.dtype, device=b2.device).t())
        vptr = ctypes.c_void_p(0)
        if values is not None:
            v = values.to(self.device, torch.float64).contiguous()
            self.values = v
            vptr = _ptr(v)
        it = ctypes.c_int(0)
        est = ctypes.c_double(0.0)
        check(self._lib.sptrsv_gb300_solve_refine(self._h, vptr, rhs, layout, _ptr(b2), _ptr(out), float(tol),
                                                  int(max_iter), ctypes.byref(it), ctypes.byref(est),
                                                  _stream_ptr(self._stream)), "solve_refine")
        x = out.reshape(b.shape) if b.dim() == 1 else out
        return x, int(it.value), float(est.value)

    def _layout_of(self, t):
        torch = _torch()
        t2 = t.reshape(-1, 1) if t.dim() == 1 else t
        if t2.is_contiguous():
            return t2, LAYOUT_ROW_MAJOR
        if t2.t().is_contiguous():
            return t2, LAYOUT_COL_MAJOR
        return t2.contiguous(), LAYOUT_ROW_MAJOR

    def solve_adjoint(self, g, x=None, *, values=None, grad_values: bool = False, out=None):
        """Solve op(L)^T lambda = g on the same analysis (reverse dependency order).
        With ``grad_values`` (needs the forward solution ``x``), also returns
        dL[e] = -sum_k lambda[row(e),k] x[col(e),k] over the stored pattern, formed by the
        same kernel as lambda. Returns (lambda, dval or None)."""
        torch = _torch()
        g2, layout = self._layout_of(g)
        rhs = int(g2.shape[1])
        dt = DTYPE_F64 if g2.dtype == torch.float64 else DTYPE_F32
        if out is None:
            out = (torch.empty_like(g2, memory_format=torch.contiguous_format) if layout == LAYOUT_ROW_MAJOR
                   else torch.empty((rhs, self.n), dtype=g2.dtype, device=g2.device).t())
        xp = ctypes.c_void_p(0)
        dval = None
        if grad_values:
            if x is None:
                raise ValueError("grad_values needs the forward solution x")
            x2, xl = self._layout_of(x)
            if xl != layout:
                x2 = x2.contiguous() if layout == LAYOUT_ROW_MAJOR else x2.t().contiguous().t()
            xp = _ptr(x2)
            dval = torch.empty(self.nnz, dtype=g2.dtype, device=g2.device)
            self._keep = x2
        vptr = ctypes.c_void_p(0)
        if values is not None:
            v = values.to(self.device).contiguous()
            self.values = v
            vptr = _ptr(v)
        check(self._lib.sptrsv_gb300_solve_adjoint(self._h, vptr, dt, rhs, layout, _ptr(g2), _ptr(out), xp,
                                                   _ptr(dval), _stream_ptr(self._stream)), "solve_adjoint")
        lam = out.reshape(g.shape) if g.dim() == 1 else out
        return lam, dval

    def grad_values(self, lam, x):
        """dL[e] = -sum_k lam[row(e),k] x[col(e),k] (standalone kernel)."""
        torch = _torch()
        l2, layout = self._layout_of(lam)
        x2, xl = self._layout_of(x)
        if xl != layout:
            x2 = x2.contiguous() if layout == LAYOUT_ROW_MAJOR else x2.t().contiguous().t()
        dt = DTYPE_F64 if l2.dtype == torch.float64 else DTYPE_F32
        dval = torch.empty(self.nnz, dtype=l2.dtype, device=l2.device)
        check(self._lib.sptrsv_gb300_grad_values(self._h, dt, int(l2.shape[1]), layout, _ptr(l2), _ptr(x2),
                                                 _ptr(dval), _stream_ptr(self._stream)), "grad_values")
        return dval

    TUNED_OPTIONS = ("SCHEDULE", "ORDER_BLOCK", "CHUNK", "STAGED", "BACKOFF_NS", "CTAS_PER_SM", "LANES", "STAGES",
                     "WARP_SYNC", "BLOCK", "SPLIT", "WSYNC_BATCH", "SMEM_TIER", "OPT", "RHS_TILE")

    def tune(self, b, values=None, reps: int = 3) -> dict:
        """Autotune the executor on this right-hand side; returns the chosen options and time."""
        torch = _torch()
        b2, layout = self._layout_of(b)
        v = (values if values is not None else self.values)
        if v is None:
            raise ValueError("tune needs the matrix values")
        v = v.to(self.device).contiguous()
        dt = DTYPE_F64 if b2.dtype == torch.float64 else DTYPE_F32
        if dt == DTYPE_F32 and v.dtype == torch.float64:
            v = v.to(torch.float32)
        x = torch.empty_like(b2)
        ms = ctypes.c_double(0.0)
        check(self._lib.sptrsv_gb300_tune(self._h, _ptr(v), dt, int(b2.shape[1]), layout, _ptr(b2), _ptr(x), int(reps),
                                          ctypes.byref(ms), _stream_ptr(self._stream)), "tune")
        self.values = v
        return {"best_ms": float(ms.value), **self.tuned_options()}

    def tuned_options(self) -> dict:
        return {k.lower(): self.get_option(getattr(_lib, "OPTION_" + k)) for k in self.TUNED_OPTIONS}

    def apply_options(self, opts: dict) -> None:
        """Apply a dict produced by tuned_options() (e.g. loaded from JSON); restage values after."""
        for k, v in opts.items():
            if k == "best_ms":
                continue
            self.set_option(getattr(_lib, "OPTION_" + k.upper()), int(v))
        if self.values is not None:
            self.set_values(self.values)

    def graph(self, b, x, *, kind: int = 0, count: int = 1):
        """Capture `count` solves (kind 0) or one refinement with `count` steps (kind 1) of the staged
        values into a CUDA graph; returns a SolveGraph to replay."""
        torch = _torch()
        b2, layout = self._layout_of(b)
        x2, _ = self._layout_of(x)
        dt = DTYPE_F64 if b2.dtype == torch.float64 else DTYPE_F32
        g = ctypes.c_void_p()
        check(self._lib.sptrsv_gb300_graph_create(self._h, int(kind), dt, int(b2.shape[1]), layout, _ptr(b2),
                                                  _ptr(x2), int(count), ctypes.byref(g), _stream_ptr(self._stream)),
              "graph_create")
        return SolveGraph(self._lib, g, (b2, x2), self._stream)

    def exec_ms(self) -> float:
        """Device time of the last executor launch (needs profile=True)."""
        ms = ctypes.c_double(0.0)
        check(self._lib.sptrsv_gb300_exec_ms(self._h, ctypes.byref(ms)), "exec_ms")
        return float(ms.value)

    def check(self) -> None:
        check(self._lib.sptrsv_gb300_check(self._h, _stream_ptr(self._stream)), "check")

    def info(self) -> dict:
        inf = _lib.Info()
        check(self._lib.sptrsv_gb300_get_info(self._h, ctypes.byref(inf)), "get_info")
        return {f: getattr(inf, f) for f, _ in _lib.Info._fields_}

    def levels(self):
        """(level_ptr [nlevels+1], level_item [n]) as int32 CUDA tensors (findlevel.h:6-69)."""
        torch = _torch()
        nl = self.info()["nlevels"]
        lp = torch.empty(nl + 1, dtype=torch.int32, device=self.device)
        li = torch.empty(max(self.n, 1), dtype=torch.int32, device=self.device)
        check(self._lib.sptrsv_gb300_levels(self._h, _ptr(lp), _ptr(li), _stream_ptr(self._stream)), "levels")
        return lp, li[: self.n]

    def csr(self):
        """(row_ptr, col_idx, src) of the analysed triangle (tranpose.h:6-43)."""
        torch = _torch()
        rp = torch.empty(self.n + 1, dtype=torch.int32, device=self.device)
        ci = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=self.device)
        src = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=self.device)
        check(self._lib.sptrsv_gb300_csr(self._h, _ptr(rp), _ptr(ci), _ptr(src), _stream_ptr(self._stream)), "csr")
        return rp, ci[: self.nnz], src[: self.nnz]

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.sptrsv_gb300_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SolveGraph:
    """A captured CUDA graph of solves; replay() launches it on the solver's stream."""

    def __init__(self, lib, handle, keep, stream):
        self._lib = lib
        self._g = handle
        self._keep = keep
        self._stream = stream

    def replay(self) -> None:
        check(self._lib.sptrsv_gb300_graph_launch(self._g, _stream_ptr(self._stream)), "graph_launch")

    def close(self) -> None:
        if self._g is not None and self._g.value:
            self._lib.sptrsv_gb300_graph_destroy(self._g)
            self._g = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

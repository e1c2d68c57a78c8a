"""Python access to the CPU oracle.

TEST INFRASTRUCTURE ONLY: what the CUDA library's results are compared with. Only the test
suite, the smoke check and the benchmark's CPU-baseline leg use this module;
the library never calls it and there is no CPU fallback.

Two implementations with one interface:
  * ``port``: liboracle.so, the C restatement in sptrsv_oracle.c (always built);
  * ``ref``:  libsptrsv_ref.so, the reference's own serial sources compiled in
    place by ``make ref`` (only where the reference checkout exists; the GPU
    host does not have it). The checkout's root directory comes from the
    environment variable SPTRSV_REFERENCE_DIR.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libsptrsv_ref.so"


def ref_sources() -> Path | None:
    """SpTRSV_cuda/ of the reference checkout named by SPTRSV_REFERENCE_DIR, if present."""
    root = os.environ.get("SPTRSV_REFERENCE_DIR")
    if not root:
        return None
    src = Path(root) / "SpTRSV_cuda"
    return src if src.exists() else None

FORWARD = 0
BACKWARD = 1


def build(ref: bool = True) -> None:
    """Compile the port (always) and the reference build (when its sources are present)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    src = ref_sources()
    if ref and src is not None:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={src}"], check=True)


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class _Impl:
    def __init__(self, path: Path, kind: str):
        self.kind = kind
        self.lib = ctypes.CDLL(str(path))
        if kind == "port":
            self._an = self.lib.oracle_analyser
            self._ex = {np.float64: self.lib.oracle_executor_f64, np.float32: self.lib.oracle_executor_f32}
            self._tr = self.lib.oracle_transpose_f64
            self._fl = self.lib.oracle_findlevel
            self._flc = self.lib.oracle_findlevel_csc
        else:
            self._an = self.lib.ref_analyser_f64
            self._ex = {np.float64: self.lib.ref_executor_f64, np.float32: self.lib.ref_executor_f32}
            self._tr = self.lib.ref_transpose_f64
            self._fl = self.lib.ref_findlevel_f64
            self._flc = self.lib.ref_findlevel_csc_f64
        for f in (self._an, self._tr, self._fl, self._flc, *self._ex.values()):
            f.restype = ctypes.c_int if f is not self._tr else None

    # sptrsv_syncfree_serialref.h:6-23
    def analyser(self, row_idx: np.ndarray, n: int) -> np.ndarray:
        row_idx = np.ascontiguousarray(row_idx, dtype=np.int32)
        out = np.zeros(max(n, 1), dtype=np.int32)
        if self.kind == "port":
            self._an(_p(row_idx), ctypes.c_int(n), ctypes.c_int(row_idx.size), _p(out))
        else:
            self._an(_p(row_idx), ctypes.c_int(n), ctypes.c_int(n), ctypes.c_int(row_idx.size), _p(out))
        return out[:n]

    # sptrsv_syncfree_serialref.h:25-108
    def executor(self, col_ptr, row_idx, val, in_degree, n, substitution, rhs, b) -> np.ndarray:
        dt = np.float32 if np.asarray(val).dtype == np.float32 else np.float64
        col_ptr = np.ascontiguousarray(col_ptr, dtype=np.int32)
        row_idx = np.ascontiguousarray(row_idx, dtype=np.int32)
        val = np.ascontiguousarray(val, dtype=dt)
        in_degree = np.ascontiguousarray(in_degree, dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=dt).reshape(-1)
        x = np.zeros(n * rhs, dtype=dt)
        self._ex[dt](_p(col_ptr), _p(row_idx), _p(val), _p(in_degree), ctypes.c_int(n), ctypes.c_int(n),
                     ctypes.c_int(substitution), ctypes.c_int(rhs), _p(b), _p(x))
        return x

    def solve(self, col_ptr, row_idx, val, n, substitution, b, rhs: int | None = None) -> np.ndarray:
        """Analyser + serial executor; b and the result are row-major n x rhs (flattened)."""
        b = np.asarray(b)
        if rhs is None:
            rhs = 1 if b.ndim == 1 else b.shape[1]
        deg = self.analyser(row_idx, n)
        x = self.executor(col_ptr, row_idx, val, deg, n, substitution, rhs, b)
        return x.reshape(b.shape) if b.ndim == 2 else x

    # tranpose.h:6-43 (CSC of the triangle -> CSR)
    def transpose(self, col_ptr, row_idx, val, n):
        col_ptr = np.ascontiguousarray(col_ptr, dtype=np.int32)
        row_idx = np.ascontiguousarray(row_idx, dtype=np.int32)
        val = np.ascontiguousarray(val, dtype=np.float64)
        nnz = row_idx.size
        out_idx = np.zeros(max(nnz, 1), dtype=np.int32)
        out_ptr = np.zeros(n + 1, dtype=np.int32)
        out_val = np.zeros(max(nnz, 1), dtype=np.float64)
        self._tr(ctypes.c_int(n), ctypes.c_int(n), ctypes.c_int(nnz), _p(col_ptr), _p(row_idx), _p(val),
                 _p(out_idx), _p(out_ptr), _p(out_val))
        return out_ptr, out_idx[:nnz], out_val[:nnz]

    # findlevel.h:6-69
    def findlevel(self, col_ptr, row_idx, n):
        row_ptr, _, _ = self.transpose(col_ptr, row_idx, np.zeros(len(row_idx)), n)
        col_ptr = np.ascontiguousarray(col_ptr, dtype=np.int32)
        row_idx = np.ascontiguousarray(row_idx, dtype=np.int32)
        nlevel = ctypes.c_int(0)
        level_ptr = np.zeros(n + 2, dtype=np.int32)
        level_item = np.zeros(max(n, 1), dtype=np.int32)
        self._fl(_p(col_ptr), _p(row_idx), _p(row_ptr), ctypes.c_int(n), ctypes.byref(nlevel), _p(level_ptr),
                 _p(level_item))
        nl = nlevel.value
        return nl, level_ptr[: nl + 1], level_item[:n]

    # findlevel.h:71-147
    def findlevel_csc(self, col_ptr, row_idx, n):
        col_ptr = np.ascontiguousarray(col_ptr, dtype=np.int32)
        row_idx = np.ascontiguousarray(row_idx, dtype=np.int32)
        nl, lo, avg, hi = (ctypes.c_int(0) for _ in range(4))
        if self.kind == "port":
            self._flc(_p(col_ptr), _p(row_idx), ctypes.c_int(n), ctypes.c_int(n), ctypes.c_int(row_idx.size),
                      ctypes.byref(nl), ctypes.byref(lo), ctypes.byref(avg), ctypes.byref(hi))
        else:
            val = np.zeros(max(row_idx.size, 1), dtype=np.float64)
            self._flc(_p(col_ptr), _p(row_idx), _p(val), ctypes.c_int(n), ctypes.c_int(n),
                      ctypes.c_int(row_idx.size), ctypes.byref(nl), ctypes.byref(lo), ctypes.byref(avg),
                      ctypes.byref(hi))
        return nl.value, lo.value, avg.value, hi.value


_CACHE: dict[str, _Impl] = {}


def port() -> _Impl:
    """The C restatement (built on demand)."""
    if "port" not in _CACHE:
        if not PORT_LIB.exists():
            build(ref=False)
        _CACHE["port"] = _Impl(PORT_LIB, "port")
    return _CACHE["port"]


def ref() -> _Impl | None:
    """The reference's own serial code, or None where it was not built."""
    if "ref" not in _CACHE:
        if not REF_LIB.exists() and ref_sources() is not None:
            build(ref=True)
        if not REF_LIB.exists():
            return None
        _CACHE["ref"] = _Impl(REF_LIB, "ref")
    return _CACHE["ref"]


def ref_read_mtx(path):
    """The reference's Matrix Market reader (mmio_highlevel.h:8-134 mmio_info and
    :137-296 mmio_data, compiled in place): (m, n, row_ptr, col_idx, val) of the CSR
    it builds (rows in file order, symmetric and hermitian storage expanded,
    duplicates kept), or None where the reference build is absent."""
    imp = ref()
    if imp is None:
        return None
    lib = imp.lib
    fn = str(path).encode()
    m, n, nnz, sym = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib.ref_mmio_info_f64.restype = ctypes.c_int
    lib.ref_mmio_data_f64.restype = ctypes.c_int
    rc = lib.ref_mmio_info_f64(ctypes.byref(m), ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(sym), fn)
    if rc != 0:
        raise ValueError(f"{path}: reference reader status {rc}")
    row_ptr = np.zeros(m.value + 1, dtype=np.int32)
    col_idx = np.zeros(max(nnz.value, 1), dtype=np.int32)
    val = np.zeros(max(nnz.value, 1), dtype=np.float64)
    rc = lib.ref_mmio_data_f64(_p(row_ptr), _p(col_idx), _p(val), fn)
    if rc != 0:
        raise ValueError(f"{path}: reference reader status {rc}")
    return m.value, n.value, row_ptr, col_idx[:nnz.value], val[:nnz.value]


def csc_spmv(col_ptr, row_idx, val, n, x):
    """b = L x in the order of main.cu:347-358 (via the port)."""
    lib = port().lib
    x = np.ascontiguousarray(x, dtype=np.float64)
    rhs = 1 if x.ndim == 1 else x.shape[1]
    b = np.zeros(x.shape, dtype=np.float64)
    lib.oracle_csc_spmv_f64(_p(np.ascontiguousarray(col_ptr, dtype=np.int32)),
                            _p(np.ascontiguousarray(row_idx, dtype=np.int32)),
                            _p(np.ascontiguousarray(val, dtype=np.float64)), ctypes.c_int(n), ctypes.c_int(n),
                            ctypes.c_int(rhs), _p(x), _p(b))
    return b


def l1_rel_err(x, x_ref) -> float:
    """sum|x - x_ref| / sum|x_ref| (sptrsv_syncfree_serialref.h:194-204)."""
    x = np.asarray(x, dtype=np.float64).ravel()
    x_ref = np.asarray(x_ref, dtype=np.float64).ravel()
    ref_ = float(np.abs(x_ref).sum())
    res = float(np.abs(x - x_ref).sum())
    return res if ref_ == 0.0 else res / ref_


def adjoint_gradient(col_ptr, row_idx, val, n, substitution, x, g):
    """Gradient of loss(x) with dloss/dx = g for x = L^-1 b: lambda = L^-T g solved by the serial
    executor on the transposed CSC (tranpose.h:6-43, opposite substitution); dL[e] = -lambda[row(e)] *
    x[col(e)] summed over right-hand sides; db = lambda. x, g: [n] or [n, rhs]."""
    imp = port()
    t_ptr, t_idx, t_val = imp.transpose(col_ptr, row_idx, val, n)
    lam = imp.solve(t_ptr, t_idx, t_val, n, 1 - substitution, g)
    lam2 = lam.reshape(n, -1)
    x2 = np.asarray(x).reshape(n, -1)
    cols = np.repeat(np.arange(n), np.diff(np.asarray(col_ptr)))
    rows = np.asarray(row_idx)
    dval = -(lam2[rows] * x2[cols]).sum(axis=1)
    return lam, dval

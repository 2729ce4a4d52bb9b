"""Host-side mirror of the reference's ``solver`` call (src/Solver.f:28-29).

``solver(ad, au, al, x, b, iax, ja, neq, nad, unsym, tol, maxit, code,
matriz, nlit)`` takes the same arguments with the same meaning as the
Fortran subroutine (numpy host arrays, Fortran 1-based indices, negated
off-diagonals) and runs the solve on the GPU through libfvcgpu's C ABI.
``x`` is updated in place.  Where the reference prints a warning and
executes STOP (non-convergence, an unsupported code/matriz pair), this
mirror raises :class:`FvcError` with the matching status instead.

:class:`Context` exposes the device-resident path: a matrix uploaded once,
device vectors (torch tensors used as plain device buffers), FP64 or mixed
precision, the reference's or the ||r||/||b|| stopping rule.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import FvcError, FvcOpts, FvcStats

CODES = {1: "PCG", 2: "BiCGSTAB", 3: "GMRES"}


def _p(a):
    return None if a is None else np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)


def make_opts(precision: str = "fp64", init: int = -1, stop_rule: int = 0,
              refine_tol: float = 0.0, inner_tol: float = 0.0, max_refine: int = 0,
              block_threads: int = 0, blocks_per_sm: int = 0,
              update_beta: int = 0, staging: int = 0, max_blocks: int = 0,
              fp32_layout: int = 0, cluster_size: int = 0) -> FvcOpts:
    o = FvcOpts()
    _lib.load().fvc_opts_default(C.byref(o))
    o.precision = {"fp64": _lib.FVC_PREC_FP64, "mixed": _lib.FVC_PREC_MIXED}[precision]
    o.init = init
    o.stop_rule = stop_rule
    o.refine_tol = refine_tol
    o.inner_tol = inner_tol
    o.max_refine = max_refine
    o.block_threads = block_threads
    o.blocks_per_sm = blocks_per_sm
    o.update_beta = update_beta
    o.staging = staging
    o.max_blocks = max_blocks
    o.fp32_layout = fp32_layout
    o.cluster_size = cluster_size
    return o


def solver(ad, au, al, x, b, iax, ja, neq, nad, unsym, tol, maxit, code, matriz, nlit=0,
           opts: FvcOpts | None = None) -> FvcStats:
    """GPU solve with the reference's argument list; returns the stats.

    Raises FvcError on non-convergence (the reference STOPs) and on the
    code/matriz pairs Solver.f rejects.
    """
    L = _lib.load()
    if x.dtype != np.float64 or not x.flags.c_contiguous:
        raise TypeError("x must be a contiguous float64 array (updated in place)")
    ad = np.ascontiguousarray(ad, np.float64)
    au = None if au is None else np.ascontiguousarray(au, np.float64)
    al = None if al is None else np.ascontiguousarray(al, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    iax = np.ascontiguousarray(iax, np.int32)
    ja = np.ascontiguousarray(ja, np.int32)
    st = FvcStats()
    o = opts if opts is not None else make_opts()
    rc = L.fvc_solver_ex(_p(ad), _p(au), _p(al), x.ctypes.data_as(C.c_void_p), _p(b), _p(iax),
                         _p(ja), int(neq), int(nad), int(bool(unsym)), float(tol), int(maxit),
                         int(code), int(matriz), C.byref(o), C.byref(st))
    if rc != _lib.FVC_OK:
        raise FvcError(rc, f"{CODES.get(code, code)} (matriz {matriz}) ended with status "
                           f"{_lib.STATUS_NAMES.get(rc, rc)} after {st.iterations} iterations")
    return st


class Context:
    """A device-resident matrix plus solver scratch (one per host thread)."""

    def __init__(self, device: int = 0, stream=None):
        self._L = _lib.load()
        self._h = C.c_void_p()
        _lib.check(self._L.fvc_context_create(C.byref(self._h), int(device)),
                   "fvc_context_create")
        if stream is not None:
            self.set_stream(stream)

    def close(self):
        if self._h:
            self._L.fvc_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream) -> None:
        """stream: a torch.cuda.Stream, a raw cudaStream_t int, or None."""
        raw = getattr(stream, "cuda_stream", stream)
        _lib.check(self._L.fvc_context_set_stream(self._h, C.c_void_p(raw or 0)),
                   "fvc_context_set_stream")

    def set_matrix(self, matriz, unsym, neq, nad, ad, au, al, iax, ja) -> None:
        self._keep = [np.ascontiguousarray(a) if a is not None else None
                      for a in (ad, au, al, iax, ja)]
        ad, au, al, iax, ja = self._keep
        _lib.check(self._L.fvc_matrix_set(self._h, int(matriz), int(bool(unsym)), int(neq),
                                          int(nad), _p(ad), _p(au), _p(al), _p(iax), _p(ja)),
                   "fvc_matrix_set")

    def update_values(self, ad, au=None, al=None) -> None:
        """New values for the structure of the last set_matrix: host numpy
        arrays or device buffers (torch CUDA float64 tensors)."""
        def ptr(a):
            if a is None:
                return None
            if hasattr(a, "data_ptr"):
                return C.c_void_p(a.data_ptr())
            return _p(a)
        _lib.check(self._L.fvc_matrix_update_values(self._h, ptr(ad), ptr(au), ptr(al)),
                   "fvc_matrix_update_values")

    def update_values_async(self, ad, au=None, al=None) -> None:
        """update_values without the wait (device arrays: capturable)."""
        def ptr(a):
            if a is None:
                return None
            if hasattr(a, "data_ptr"):
                return C.c_void_p(a.data_ptr())
            return _p(a)
        _lib.check(self._L.fvc_matrix_update_values_async(self._h, ptr(ad), ptr(au), ptr(al)),
                   "fvc_matrix_update_values_async")

    def info(self) -> dict:
        n, slots, nnz, ns = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        _lib.check(self._L.fvc_matrix_info(self._h, C.byref(n), C.byref(slots), C.byref(nnz),
                                           C.byref(ns)), "fvc_matrix_info")
        return {"n": n.value, "slots": slots.value, "nnz_off": nnz.value, "nslices": ns.value}

    def solve(self, code: int, b_dev, x_dev, tol: float, maxit: int,
              opts: FvcOpts | None = None, raise_on_error: bool = True) -> FvcStats:
        """b_dev, x_dev: device buffers (torch CUDA float64 tensors or raw
        device addresses).  x_dev is the initial guess and the result."""
        st = FvcStats()
        o = opts if opts is not None else make_opts()
        rc = self._L.fvc_solve(self._h, int(code), C.c_void_p(_addr(b_dev)),
                               C.c_void_p(_addr(x_dev)), float(tol), int(maxit), C.byref(o),
                               C.byref(st))
        if raise_on_error and rc != _lib.FVC_OK:
            raise FvcError(rc, f"{CODES.get(code, code)} ended with status "
                               f"{_lib.STATUS_NAMES.get(rc, rc)}")
        st.status = rc
        return st

    def solve_async(self, code: int, b_dev, x_dev, tol: float, maxit: int, status_dev,
                    opts: FvcOpts | None = None) -> None:
        """Enqueues an FP64 solve on the context's stream without waiting
        (capturable into a CUDA graph).  status_dev: a device int32 buffer of
        4 entries that receives status, iterations, inner iterations and the
        timeout flag when the solve has run."""
        o = opts if opts is not None else make_opts()
        _lib.check(self._L.fvc_solve_async(self._h, int(code), C.c_void_p(_addr(b_dev)),
                                           C.c_void_p(_addr(x_dev)), float(tol), int(maxit),
                                           C.byref(o), C.c_void_p(_addr(status_dev))),
                   "fvc_solve_async")

    def solve_transposed(self, b_dev, x_dev, tol: float, maxit: int,
                         opts: FvcOpts | None = None, raise_on_error: bool = True) -> FvcStats:
        """A^T x = b by BiCGSTAB over this context's matrix (no transposed
        copy); device buffers as in solve."""
        st = FvcStats()
        o = opts if opts is not None else make_opts()
        rc = self._L.fvc_solve_transposed(self._h, 2, C.c_void_p(_addr(b_dev)),
                                          C.c_void_p(_addr(x_dev)), float(tol), int(maxit),
                                          C.byref(o), C.byref(st))
        if raise_on_error and rc != _lib.FVC_OK:
            raise FvcError(rc, f"transposed BiCGSTAB ended with status "
                               f"{_lib.STATUS_NAMES.get(rc, rc)}")
        st.status = rc
        return st

    def autotune(self, code: int, precision: str = "fp64", trial_its: int = 50):
        """The fastest launch shape for this matrix and method (fvc_autotune):
        (FvcOpts to pass to solve, microseconds per iteration)."""
        o = FvcOpts()
        us = C.c_double()
        prec = {"fp64": 0, "mixed": 1}[precision]
        _lib.check(self._L.fvc_autotune(self._h, int(code), prec, int(trial_its), C.byref(o),
                                        C.byref(us)), "fvc_autotune")
        return o, us.value

    def solve_batched(self, row_start, b_dev, x_dev, tol: float, maxit: int,
                      opts: FvcOpts | None = None, raise_on_error: bool = True,
                      codes=None, tols=None, its_hint=None):
        """Batched solves of the block-diagonal matrix on this context (see
        pack_block_diagonal): one persistent launch, each system on its own
        blocks with its own stopping test.  codes: per system 1 (PCG, the
        default) or 2 (BiCGSTAB); tols: per-system tolerances (default tol);
        its_hint: expected iterations per system, for the share of blocks.
        Returns (status, [FvcStats] per system)."""
        rs = np.ascontiguousarray(row_start, np.int32)
        nsys = rs.size - 1
        st = (FvcStats * nsys)()
        o = opts if opts is not None else make_opts()
        cd = None if codes is None else np.ascontiguousarray(codes, np.int32)
        td = None if tols is None else np.ascontiguousarray(tols, np.float64)
        hd = None if its_hint is None else np.ascontiguousarray(its_hint, np.float64)
        for arr in (cd, td, hd):
            if arr is not None and arr.size != nsys:
                raise ValueError("codes, tols and its_hint need one entry per system")
        ptr = lambda arr: None if arr is None else arr.ctypes.data_as(C.c_void_p)
        rc = self._L.fvc_solve_batched_ex(
            self._h, nsys, rs.ctypes.data_as(C.c_void_p), ptr(cd), ptr(td), ptr(hd),
            C.c_void_p(_addr(b_dev)), C.c_void_p(_addr(x_dev)), float(tol), int(maxit),
            C.byref(o), C.cast(st, C.c_void_p))
        if raise_on_error and rc != _lib.FVC_OK:
            raise FvcError(rc, f"batched solve ended with status {_lib.STATUS_NAMES.get(rc, rc)}")
        return rc, list(st)

    def trace(self, max_records: int = 256):
        """(iterations, rel. residuals) at the residual replacements of the
        last mixed-precision CG solve."""
        its = np.zeros(max_records, np.int32)
        rel = np.zeros(max_records, np.float64)
        k = self._L.fvc_solve_trace(self._h, max_records, its.ctypes.data_as(C.c_void_p),
                                    rel.ctypes.data_as(C.c_void_p))
        if k < 0:
            raise FvcError(-k, "fvc_solve_trace failed")
        return its[:k], rel[:k]

    def history(self, max_values: int = 16384) -> np.ndarray:
        """Recursive ||r||/||b|| after each iteration of the last
        mixed-precision CG solve."""
        out = np.zeros(max_values, np.float32)
        k = self._L.fvc_solve_history(self._h, max_values, out.ctypes.data_as(C.c_void_p))
        if k < 0:
            raise FvcError(-k, "fvc_solve_history failed")
        return out[:k]

    def spmv(self, x_dev, y_dev) -> None:
        _lib.check(self._L.fvc_spmv(self._h, C.c_void_p(_addr(x_dev)), C.c_void_p(_addr(y_dev))),
                   "fvc_spmv")

    def spmv_fast(self, x_dev, y_dev) -> None:
        _lib.check(self._L.fvc_spmv_fast(self._h, C.c_void_p(_addr(x_dev)),
                                         C.c_void_p(_addr(y_dev))), "fvc_spmv_fast")

    def spmv_f32(self, x_dev, y_dev) -> None:
        _lib.check(self._L.fvc_spmv_f32(self._h, C.c_void_p(_addr(x_dev)),
                                        C.c_void_p(_addr(y_dev))), "fvc_spmv_f32")


def _addr(t) -> int:
    if hasattr(t, "data_ptr"):
        if not t.is_cuda or not t.is_contiguous():
            raise ValueError("device buffers must be contiguous CUDA tensors")
        return int(t.data_ptr())
    return int(t)


_LOG_FN = C.CFUNCTYPE(None, C.c_char_p, C.c_void_p)
_log_keep = None


def set_solver_log(fn=None) -> None:
    """fn(line: str) receives, after every solve, the line the reference
    writes to its unit-13 solver log (src/Iterativos.f:91-93); None stops."""
    global _log_keep
    L = _lib.load()
    if fn is None:
        L.fvc_set_solver_log(None, None)
        _log_keep = None
        return
    _log_keep = _LOG_FN(lambda line, user: fn(line.decode()))
    L.fvc_set_solver_log(C.cast(_log_keep, C.c_void_p), None)


def format_solver_log(code: int, iterations: int, energy: float, tol: float) -> str:
    """The reference's unit-13 line for the given values."""
    buf = C.create_string_buffer(128)
    n = _lib.load().fvc_format_solver_log(int(code), int(iterations), float(energy), float(tol),
                                          buf, 128)
    if n < 0:
        raise FvcError(-n, "fvc_format_solver_log failed")
    return buf.value.decode()


def kernel_launches() -> int:
    return int(_lib.load().fvc_kernel_launches())


def pack_block_diagonal(systems):
    """Packs CSRD systems (each a dict with ad, au, ia, ja: 1-based, negated
    off-diagonals, as src/Datastruct.f builds them for matriz 1) into one
    block-diagonal CSRD matrix whose systems start at multiples of 32 rows,
    as fvc_solve_batched requires; the rows in between are identity rows.
    Returns dict(ad, au, ia, ja, neq, nad, row_start, rows): rows[s] is the
    index array of system s's rows in the packed vectors."""
    starts, rows, n = [], [], 0
    for s in systems:
        k = int(s["ad"].size)
        starts.append(n)
        rows.append(np.arange(n, n + k))
        n += (k + 31) // 32 * 32
    row_start = np.array(starts + [n], np.int32)
    ad = np.ones(n)
    nnz = [np.diff(np.asarray(s["ia"])) for s in systems]
    counts = np.zeros(n, np.int64)
    for r, c in zip(rows, nnz):
        counts[r] = c
    ia = np.ones(n + 1, np.int64)
    ia[1:] = 1 + np.cumsum(counts)
    ja = np.empty(int(counts.sum()), np.int32)
    au = np.empty(ja.size)
    for s, r, st in zip(systems, rows, starts):
        ad[r] = s["ad"]
        lo, hi = ia[r[0]] - 1, ia[r[-1] + 1] - 1
        ja[lo:hi] = np.asarray(s["ja"][: hi - lo]) + st
        au[lo:hi] = s["au"][: hi - lo]
    return dict(ad=ad, au=au, ia=ia.astype(np.int32), ja=ja, neq=n, nad=int(ja.size),
                row_start=row_start, rows=rows)

"""GB300 (sm_103a) recursive QR / Cholesky — Python host side.

The compute path is the shared library `later_gb300/_lib/liblater_gb300.so`
(hand-written CUDA for sm_103a behind the C ABI of `include/later_c.h`). This
module binds that ABI with ctypes and mirrors the reference's entry points
(`later_rgsqrf`, ... of LATER's include/LATER.h) for torch CUDA tensors in
column-major layout: a (m, n) tensor with stride (1, lda).

There is no CPU or PyTorch fallback: if the library is missing, every entry
point raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

from . import build as _build

__all__ = [
    "LaterError", "Options", "PREC", "lib", "colmajor", "empty_colmajor",
    "later_rgsqrf", "rgsqrf_bufsize", "later_rgsqrf_host", "later_oc_rgsqrf", "oc_rgsqrf_bytes",
    "later_rhouqr", "rhouqr_bufsize", "later_ormqr", "later_bhouqr",
    "bhouqr_bufsize", "later_ormqr2", "later_qdwh_polar", "qdwh_bufsize", "later_sy2sb",
    "sy2sb_bufsize", "later_rsyrk", "later_rtrsm",
    "later_rtrmm", "later_rpotrf", "blas3_bufsize",
    "spd_solve", "ls_solve", "BatchedQR", "LsServer", "gemm16", "convert16", "device_status", "wait_selftest", "launch_count", "trace_begin",
    "trace_end",
]

PREC = {"fp16": 0, "bf16": 1, "split3": 2, "split2": 3}
STATUS = {0: "ok", 1: "invalid argument", 2: "workspace too small", 3: "CUDA runtime error",
          4: "device wait timed out", 5: "not supported", 6: "value outside the FP16 operand range",
          7: "non-positive pivot"}


class LaterError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)} (status {status})")


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("cgs2", ctypes.c_int), ("leaf", ctypes.c_int),
                ("panel", ctypes.c_int), ("timeout_cycles", ctypes.c_longlong)]

    @classmethod
    def make(cls, precision="fp16", cgs2=False, leaf=128, timeout_cycles=0, panel=0) -> "Options":
        p = PREC[precision] if isinstance(precision, str) else int(precision)
        pn = {"fused": 0, "mgs": 1, "wide": 2}[panel] if isinstance(panel, str) else int(panel)
        return cls(p, int(bool(cgs2)), int(leaf), pn, int(timeout_cycles))


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("factor_precision", ctypes.c_int), ("backward_error", ctypes.c_double)]


class QrItem(ctypes.Structure):
    _fields_ = [("A", ctypes.c_void_p), ("R", ctypes.c_void_p), ("lda", ctypes.c_int64), ("ldr", ctypes.c_int64),
                ("m", ctypes.c_int), ("n", ctypes.c_int)]


class LsRequest(ctypes.Structure):
    _fields_ = [("m", ctypes.c_int), ("n", ctypes.c_int), ("nrhs", ctypes.c_int), ("reserved", ctypes.c_int),
                ("A", ctypes.c_void_p), ("B", ctypes.c_void_p), ("X", ctypes.c_void_p),
                ("lda", ctypes.c_int), ("ldb", ctypes.c_int), ("ldx", ctypes.c_int), ("reserved2", ctypes.c_int)]


class LsResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int), ("slot", ctypes.c_int),
                ("reserved", ctypes.c_int), ("backward_error", ctypes.c_double), ("submit_ms", ctypes.c_double),
                ("queue_ms", ctypes.c_double), ("service_ms", ctypes.c_double), ("latency_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("reserved")}


class Trace(ctypes.Structure):
    _fields_ = [("gemm_flops", ctypes.c_double), ("gemm_ms", ctypes.c_double), ("gemm_launches", ctypes.c_int64),
                ("top_gemm_flops", ctypes.c_double), ("top_gemm_ms", ctypes.c_double),
                ("panel_ms", ctypes.c_double), ("panel_launches", ctypes.c_int64),
                ("leaf_gemm_flops", ctypes.c_double), ("leaf_gemm_ms", ctypes.c_double),
                ("leaf_gemm_launches", ctypes.c_int64), ("other_ms", ctypes.c_double),
                ("other_launches", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None
_vp, _i, _i64, _f = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float
_SIGS = {
    "later_c_default_options": (None, [ctypes.POINTER(Options)]),
    "later_c_status_string": (ctypes.c_char_p, [_i]),
    "later_c_device_status": (_i, [_vp]),
    "later_c_wait_selftest": (_i, [_vp, ctypes.c_longlong]),
    "later_c_rgsqrf_bufsize": (_i, [_i, _i, ctypes.POINTER(Options), ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "later_c_rgsqrf": (_i, [_vp, _i, _i, _vp, _i, _vp, _i, _vp, _i64, _vp, _i64, ctypes.POINTER(Options)]),
    "later_c_gemm16": (_i, [_vp, ctypes.c_char, ctypes.c_char, _i, _i, _i, _f, _vp, _i, _vp, _i, _f, _vp, _i,
                            _vp, _i, _i, _vp, _i64]),
    "later_c_convert": (_i, [_vp, _i, _i, _vp, _i, _vp, _vp, _i, _i]),
    "later_c_rhouqr_bufsize": (_i, [_i, _i, ctypes.POINTER(Options), ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "later_c_rhouqr": (_i, [_vp, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i64, _vp, _i64, ctypes.POINTER(Options)]),
    "later_c_ormqr": (_i, [_vp, _i, _i, _vp, _i, _vp, _i, _vp, _i64]),
    "later_c_oc_rgsqrf_bufsize": (_i, [_i, _i, ctypes.POINTER(Options), ctypes.POINTER(_i64)]),
    "later_c_oc_rgsqrf": (_i, [_vp, _i, _i, _vp, _i, _vp, _i, _i, _vp, _i64, ctypes.POINTER(Options)]),
    "later_c_rgsqrf_host": (_i, [_vp, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i64, _vp, _i64,
                                 ctypes.POINTER(Options)]),
    "later_c_sy2sb_bufsize": (_i, [_i, _i, ctypes.POINTER(Options), ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "later_c_sy2sb": (_i, [_vp, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i64, _vp, _i64, ctypes.POINTER(Options)]),
    "later_c_qdwh_bufsize": (_i, [_i, _i, ctypes.POINTER(Options), ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "later_c_qdwh_polar": (_i, [_vp, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i64, _vp, _i64,
                                ctypes.POINTER(Options), ctypes.c_double, _i, ctypes.c_double, _i,
                                ctypes.POINTER(_i)]),
    "later_c_bhouqr_bufsize": (_i, [_i, _i, ctypes.POINTER(Options), ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "later_c_bhouqr": (_i, [_vp, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i64, _vp, _i64, ctypes.POINTER(Options)]),
    "later_c_blas3_bufsize": (_i, [ctypes.c_char, ctypes.c_char, _i, _i, ctypes.POINTER(Options),
                                   ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "later_c_rsyrk": (_i, [_vp, _i, _i, _f, _vp, _i, _f, _vp, _i, _vp, _i64, _vp, _i64, ctypes.POINTER(Options)]),
    "later_c_rtrsm": (_i, [_vp, ctypes.c_char, ctypes.c_char, ctypes.c_char, _i, _i, _vp, _i, _vp, _i, _vp, _i64,
                           _vp, _i64, ctypes.POINTER(Options)]),
    "later_c_rtrmm": (_i, [_vp, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i64, _vp, _i64, ctypes.POINTER(Options)]),
    "later_c_rpotrf": (_i, [_vp, ctypes.c_char, _i, _vp, _i, _vp, _i64, _vp, _i64, ctypes.POINTER(Options)]),
    "later_c_spd_solve_bufsize": (_i, [_i, _i, ctypes.POINTER(Options), ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "later_c_ls_solve_bufsize": (_i, [_i, _i, _i, ctypes.POINTER(Options), ctypes.POINTER(_i64),
                                      ctypes.POINTER(_i64)]),
    "later_c_batched_plan_bytes": (_i64, [_i]),
    "later_c_batched_qr_plan": (_i, [_vp, _i, _vp, _vp, _i64]),
    "later_c_batched_qr_run": (_i, [_vp, _i, _vp, _vp, _vp, _i]),
    "later_c_ls_server_create": (_vp, [_i, _i, _i64, ctypes.POINTER(Options), _i, ctypes.c_double]),
    "later_c_ls_server_submit": (_i64, [_vp, ctypes.POINTER(LsRequest)]),
    "later_c_ls_server_wait": (_i, [_vp, _i64, ctypes.POINTER(LsResult)]),
    "later_c_ls_server_hbm_in_use": (_i64, [_vp]),
    "later_c_ls_server_hbm_peak": (_i64, [_vp]),
    "later_c_ls_server_destroy": (None, [_vp]),
    "later_c_launch_count": (ctypes.c_uint64, []),
    "later_c_trace_begin": (None, []),
    "later_c_trace_end": (_i, [_vp]),
}


def lib_path() -> Path:
    return _build.LIB


def lib() -> ctypes.CDLL:
    """Loads the shared library (building it first if the sources are newer)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if os.environ.get("LATER_GB300_NO_BUILD") != "1":
            path = _build.build()
        if not path.exists():
            raise RuntimeError(f"later_gb300: shared library {path} is missing; run later_gb300.build.build()")
        l = ctypes.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


# ------------------------------------------------------------------ helpers
def colmajor(t):
    """Column-major copy of a 2-D tensor (stride (1, rows))."""
    return t.t().contiguous().t()


def empty_colmajor(m, n, dtype=None, device="cuda", ld=None):
    import torch
    ld = m if ld is None else ld
    buf = torch.empty((n, ld), dtype=dtype or torch.float32, device=device)
    return buf.t()[:m, :]


def _ld(t, name) -> int:
    if t.dim() != 2 or t.stride(0) != 1:
        raise ValueError(f"{name} must be a column-major 2-D tensor (stride(0) == 1)")
    return max(t.stride(1), t.shape[0], 1)


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _check(status: int, where: str):
    if status != 0:
        raise LaterError(status, where)


def device_status(stream=None) -> int:
    """Synchronises the stream and returns (and clears) the device status word."""
    return lib().later_c_device_status(_stream(stream))


def wait_selftest(timeout_cycles=0, stream=None):
    """Enqueues the bounded-wait self-check: its waits run out after timeout_cycles and the next
    device_status() returns 4 (LATER_ERR_TIMEOUT)."""
    _check(lib().later_c_wait_selftest(_stream(stream), int(timeout_cycles)), "wait_selftest")


def launch_count() -> int:
    """Cumulative number of kernels the library has launched."""
    return int(lib().later_c_launch_count())


def trace_begin():
    lib().later_c_trace_begin()


def trace_end() -> dict:
    t = Trace()
    _check(lib().later_c_trace_end(ctypes.byref(t)), "trace_end")
    return t.as_dict()


def rgsqrf_bufsize(m, n, precision="fp16", cgs2=False, leaf=128):
    o = Options.make(precision, cgs2, leaf)
    lw, lh = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().later_c_rgsqrf_bufsize(m, n, ctypes.byref(o), ctypes.byref(lw), ctypes.byref(lh)), "rgsqrf_bufsize")
    return lw.value, lh.value


def later_rgsqrf(A, R=None, work=None, hwork=None, *, precision="fp16", cgs2=False, leaf=128, timeout_cycles=0,
                 stream=None, panel="fused"):
    """Recursive Gram-Schmidt QR in place: A (m x n, column-major FP32 CUDA) becomes Q; returns R.

    Mirrors LATER's `later_rgsqrf(ctxt, m, n, A, lda, R, ldr, work, lwork, hwork, lhwork)`
    (include/LATER.h:39). Workspaces are allocated here when not given.
    """
    import torch
    m, n = A.shape
    lda = _ld(A, "A")
    if R is None:
        R = empty_colmajor(n, n, device=A.device)
    ldr = _ld(R, "R")
    lw, lh = rgsqrf_bufsize(m, n, precision, cgs2, leaf)
    if work is None:
        work = torch.empty(lw, dtype=torch.float32, device=A.device)
    if hwork is None:
        hwork = torch.empty(lh, dtype=torch.float16, device=A.device)
    o = Options.make(precision, cgs2, leaf, timeout_cycles, panel)
    _check(lib().later_c_rgsqrf(_stream(stream), m, n, A.data_ptr(), lda, R.data_ptr(), ldr, work.data_ptr(),
                                work.numel(), hwork.data_ptr(), hwork.numel(), ctypes.byref(o)), "later_rgsqrf")
    return R


def later_rgsqrf_host(hA, hQ, hR, A, R, work=None, hwork=None, *, precision="fp16", cgs2=False, leaf=128,
                      panel="fused", stream=None):
    """rgsqrf with host buffers: hA (pinned, column-major m x n) in; Q into hQ (may be hA) and the upper
    triangle of R into hR, copied in and out in column chunks overlapped with the factorisation. A and R
    are the device buffers it runs in. Asynchronous on `stream` like the other calls."""
    import torch
    m, n = hA.shape
    lw, lh = rgsqrf_bufsize(m, n, precision, cgs2, leaf)
    if work is None:
        work = torch.empty(lw, dtype=torch.float32, device=A.device)
    if hwork is None:
        hwork = torch.empty(lh, dtype=torch.float16, device=A.device)
    o = Options.make(precision, cgs2, leaf, 0, panel)
    _check(lib().later_c_rgsqrf_host(_stream(stream), m, n, hA.data_ptr(), _ld(hA, "hA"), hQ.data_ptr(),
                                     _ld(hQ, "hQ"), hR.data_ptr(), _ld(hR, "hR"), A.data_ptr(), _ld(A, "A"),
                                     R.data_ptr(), _ld(R, "R"), work.data_ptr(), work.numel(), hwork.data_ptr(),
                                     hwork.numel(), ctypes.byref(o)), "later_rgsqrf_host")


def oc_rgsqrf_bytes(m, panel, precision="split2", cgs2=False):
    o = Options.make(precision, cgs2)
    b = ctypes.c_int64()
    _check(lib().later_c_oc_rgsqrf_bufsize(m, panel, ctypes.byref(o), ctypes.byref(b)), "oc_rgsqrf_bufsize")
    return b.value


def later_oc_rgsqrf(hA, hR, dev, panel=0, *, precision="split2", cgs2=False, stream=None):
    """Out-of-core QR: hA (host, column-major) becomes Q, hR receives R; `dev` is a device byte buffer
    (torch uint8 tensor) the factorisation runs through (include/LATER.h:49-51 later_oc_qr_rec / _blk)."""
    m, n = hA.shape
    o = Options.make(precision, cgs2)
    _check(lib().later_c_oc_rgsqrf(_stream(stream), m, n, hA.data_ptr(), _ld(hA, "hA"), hR.data_ptr(),
                                   _ld(hR, "hR"), int(panel), dev.data_ptr(), dev.numel() * dev.element_size(),
                                   ctypes.byref(o)), "later_oc_rgsqrf")


def rhouqr_bufsize(m, n, precision="fp16"):
    o = Options.make(precision)
    lw, lh = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().later_c_rhouqr_bufsize(m, n, ctypes.byref(o), ctypes.byref(lw), ctypes.byref(lh)), "rhouqr_bufsize")
    return lw.value, lh.value


def later_rhouqr(A, W=None, R=None, work=None, hwork=None, *, precision="fp16", timeout_cycles=0, stream=None):
    """Recursive Householder QR: A becomes Y; returns (W, R) with Q = I - W Y^T.

    Mirrors LATER's `later_rhouqr(ctxt, m, n, A, lda, W, ldw, R, ldr, work, lwork, hwork, lhwork, U)`
    (include/LATER.h:41).
    """
    import torch
    m, n = A.shape
    if W is None:
        W = empty_colmajor(m, n, device=A.device)
    if R is None:
        R = empty_colmajor(n, n, device=A.device)
    lw, lh = rhouqr_bufsize(m, n, precision)
    if work is None:
        work = torch.empty(lw, dtype=torch.float32, device=A.device)
    if hwork is None:
        hwork = torch.empty(lh, dtype=torch.float16, device=A.device)
    o = Options.make(precision, False, 128, timeout_cycles)
    _check(lib().later_c_rhouqr(_stream(stream), m, n, A.data_ptr(), _ld(A, "A"), W.data_ptr(), _ld(W, "W"),
                                R.data_ptr(), _ld(R, "R"), work.data_ptr(), work.numel(), hwork.data_ptr(),
                                hwork.numel(), ctypes.byref(o)), "later_rhouqr")
    return W, R


def bhouqr_bufsize(m, n, precision="fp16"):
    o = Options.make(precision)
    lw, lh = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().later_c_bhouqr_bufsize(m, n, ctypes.byref(o), ctypes.byref(lw), ctypes.byref(lh)), "bhouqr_bufsize")
    return lw.value, lh.value


def later_bhouqr(A, W=None, R=None, work=None, hwork=None, *, precision="split3", timeout_cycles=0, stream=None):
    """Blocked Householder QR over 128-column rhouqr panels: A becomes Y; returns (W, R), Q = I - W Y^T.

    Mirrors LATER's `later_bhouqr(m, n, A, lda, W, ldw, R, ldr, work, lwork, hwork, lhwork, U)`
    (include/LATER.h:45); the reference's FP32 updates correspond to precision "split3".
    """
    import torch
    m, n = A.shape
    if W is None:
        W = empty_colmajor(m, n, device=A.device)
    if R is None:
        R = empty_colmajor(n, n, device=A.device)
    lw, lh = bhouqr_bufsize(m, n, precision)
    if work is None:
        work = torch.empty(lw, dtype=torch.float32, device=A.device)
    if hwork is None:
        hwork = torch.empty(lh, dtype=torch.float16, device=A.device)
    o = Options.make(precision, False, 128, timeout_cycles)
    _check(lib().later_c_bhouqr(_stream(stream), m, n, A.data_ptr(), _ld(A, "A"), W.data_ptr(), _ld(W, "W"),
                                R.data_ptr(), _ld(R, "R"), work.data_ptr(), work.numel(), hwork.data_ptr(),
                                hwork.numel(), ctypes.byref(o)), "later_bhouqr")
    return W, R


def qdwh_bufsize(m, n, precision="split3"):
    o = Options.make(precision)
    lw, lh = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().later_c_qdwh_bufsize(m, n, ctypes.byref(o), ctypes.byref(lw), ctypes.byref(lh)), "qdwh_bufsize")
    return lw.value, lh.value


def later_qdwh_polar(A, U=None, H=None, *, precision="split3", l0=0.0, symmetric=False, tol=1e-6, max_iter=10,
                     work=None, hwork=None, stream=None):
    """Polar decomposition A = U H by QDWH; returns (U, H, iterations).

    Mirrors LATER's `later_qdwh_polar(ctxt, n, A, lda, H, ldh, tmpA, work, hwork)` (include/LATER.h:70) with
    the input A (m x n, m >= n) read only; see later_c.h for the options.
    """
    import torch
    m, n = A.shape
    if U is None:
        U = empty_colmajor(m, n, device=A.device)
    if H is None:
        H = empty_colmajor(n, n, device=A.device)
    lw, lh = qdwh_bufsize(m, n, precision)
    if work is None:
        work = torch.empty(lw, dtype=torch.float32, device=A.device)
    if hwork is None:
        hwork = torch.empty(lh, dtype=torch.float16, device=A.device)
    o = Options.make(precision)
    it = ctypes.c_int(0)
    _check(lib().later_c_qdwh_polar(_stream(stream), m, n, A.data_ptr(), _ld(A, "A"), U.data_ptr(), _ld(U, "U"),
                                    H.data_ptr(), _ld(H, "H"), work.data_ptr(), work.numel(), hwork.data_ptr(),
                                    hwork.numel(), ctypes.byref(o), float(l0), int(bool(symmetric)), float(tol),
                                    int(max_iter), ctypes.byref(it)), "later_qdwh_polar")
    return U, H, it.value


def sy2sb_bufsize(n, nb=128, precision="split3"):
    o = Options.make(precision)
    lw, lh = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().later_c_sy2sb_bufsize(n, nb, ctypes.byref(o), ctypes.byref(lw), ctypes.byref(lh)), "sy2sb_bufsize")
    return lw.value, lh.value


def later_sy2sb(A, nb=128, *, precision="split3", Y=None, W=None, reflectors=True, work=None, hwork=None,
                stream=None):
    """Symmetric to band reduction in place: A (n x n, both triangles) becomes B = Q^T A Q with bandwidth nb.
    Returns (Y, W) with Q = prod_i (I - W_i Y_i^T) per block column (None, None without reflectors).

    Mirrors LATER's `ssytrd_sy2sb` / `later_sy2sb_rec` (include/LATER.h:72-74).
    """
    import torch
    n = A.shape[0]
    if reflectors:
        Y = Y if Y is not None else empty_colmajor(n, n, device=A.device)
        W = W if W is not None else empty_colmajor(n, n, device=A.device)
    lw, lh = sy2sb_bufsize(n, nb, precision)
    if work is None:
        work = torch.empty(lw, dtype=torch.float32, device=A.device)
    if hwork is None:
        hwork = torch.empty(lh, dtype=torch.float16, device=A.device)
    o = Options.make(precision)
    _check(lib().later_c_sy2sb(_stream(stream), n, nb, A.data_ptr(), _ld(A, "A"),
                               Y.data_ptr() if Y is not None else None, _ld(Y, "Y") if Y is not None else n,
                               W.data_ptr() if W is not None else None, _ld(W, "W") if W is not None else n,
                               work.data_ptr(), work.numel(), hwork.data_ptr(), hwork.numel(), ctypes.byref(o)),
           "later_sy2sb")
    return Y, W


def later_ormqr2(W, Y, work=None, stream=None):
    """Explicit Q = I - W Y^T from later_bhouqr's output, written over W (include/LATER.h:47)."""
    return later_ormqr(W, Y, work=work, stream=stream)


def later_ormqr(W, Y, work=None, stream=None):
    """Explicit Q = I - W Y^T (first n columns) written over W (include/LATER.h:43)."""
    import torch
    m, n = W.shape
    if work is None:
        work = torch.empty(m * n, dtype=torch.float32, device=W.device)
    _check(lib().later_c_ormqr(_stream(stream), m, n, W.data_ptr(), _ld(W, "W"), Y.data_ptr(), _ld(Y, "Y"),
                               work.data_ptr(), work.numel()), "later_ormqr")
    return W


def blas3_bufsize(op, m, n, side="l", precision="fp16"):
    o = Options.make(precision)
    lw, lh = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().later_c_blas3_bufsize(op.encode(), side.encode(), m, n, ctypes.byref(o), ctypes.byref(lw),
                                       ctypes.byref(lh)), "blas3_bufsize")
    return lw.value, lh.value


def _b3_ws(op, m, n, side, precision, device, work, hwork):
    import torch
    lw, lh = blas3_bufsize(op, m, n, side, precision)
    if work is None:
        work = torch.empty(lw, dtype=torch.float32, device=device)
    if hwork is None:
        hwork = torch.empty(max(lh, 8), dtype=torch.float16, device=device)
    return work, hwork


def later_rsyrk(n, k, alpha, A, beta, C, *, precision="fp16", work=None, hwork=None, stream=None):
    """C <- alpha A A^T + beta C, lower triangle (include/LATER.h:62)."""
    work, hwork = _b3_ws("s", n, k, "l", precision, C.device, work, hwork)
    o = Options.make(precision)
    _check(lib().later_c_rsyrk(_stream(stream), n, k, alpha, A.data_ptr(), _ld(A, "A"), beta, C.data_ptr(),
                               _ld(C, "C"), work.data_ptr(), work.numel(), hwork.data_ptr(), hwork.numel(),
                               ctypes.byref(o)), "later_rsyrk")
    return C


def later_rtrsm(uplo, leri, trans, m, n, A, B, *, precision="fp16", work=None, hwork=None, stream=None):
    """In-place triangular solve, ('l','l','n') or ('l','r','t') (include/LATER.h:60)."""
    work, hwork = _b3_ws("t", m, n, leri, precision, B.device, work, hwork)
    o = Options.make(precision)
    _check(lib().later_c_rtrsm(_stream(stream), uplo.encode(), leri.encode(), trans.encode(), m, n, A.data_ptr(),
                               _ld(A, "A"), B.data_ptr(), _ld(B, "B"), work.data_ptr(), work.numel(),
                               hwork.data_ptr(), hwork.numel(), ctypes.byref(o)), "later_rtrsm")
    return B


def later_rtrmm(m, n, A, B, C, *, precision="fp16", work=None, hwork=None, stream=None):
    """C = A B, A lower triangular (include/LATER.h:64)."""
    work, hwork = _b3_ws("m", m, n, "l", precision, C.device, work, hwork)
    o = Options.make(precision)
    _check(lib().later_c_rtrmm(_stream(stream), m, n, A.data_ptr(), _ld(A, "A"), B.data_ptr(), _ld(B, "B"),
                               C.data_ptr(), _ld(C, "C"), work.data_ptr(), work.numel(), hwork.data_ptr(),
                               hwork.numel(), ctypes.byref(o)), "later_rtrmm")
    return C


def later_rpotrf(uplo, n, A, *, precision="fp16", work=None, hwork=None, stream=None):
    """Lower Cholesky in place (include/LATER.h:80)."""
    work, hwork = _b3_ws("p", n, n, "l", precision, A.device, work, hwork)
    o = Options.make(precision)
    _check(lib().later_c_rpotrf(_stream(stream), uplo.encode(), n, A.data_ptr(), _ld(A, "A"), work.data_ptr(),
                                work.numel(), hwork.data_ptr(), hwork.numel(), ctypes.byref(o)), "later_rpotrf")
    return A


def _solve_ws(lw, lh, device, work, hwork):
    import torch
    if work is None:
        work = torch.empty(lw, dtype=torch.float32, device=device)
    if hwork is None:
        hwork = torch.empty(max(lh, 8), dtype=torch.float16, device=device)
    return work, hwork


def _bind_solver(name):
    fn = getattr(lib(), name)
    fn.restype = _i
    if name == "later_c_spd_solve":
        fn.argtypes = [_vp, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i64, _vp, _i64, ctypes.POINTER(Options), _i,
                       ctypes.c_double, ctypes.POINTER(SolveInfo)]
    else:
        fn.argtypes = [_vp, _i, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp, _i64, _vp, _i64, ctypes.POINTER(Options), _i,
                       ctypes.c_double, ctypes.POINTER(SolveInfo)]
    return fn


def spd_solve(A, B, *, precision="fp16", max_iter=30, tol=1e-12, work=None, hwork=None, stream=None):
    """SPD solve with FP64 refinement; returns (X (FP64, column-major), info dict)."""
    import torch
    n, k = B.shape
    o = Options.make(precision)
    lw, lh = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().later_c_spd_solve_bufsize(n, k, ctypes.byref(o), ctypes.byref(lw), ctypes.byref(lh)), "bufsize")
    work, hwork = _solve_ws(lw.value, lh.value, A.device, work, hwork)
    X = empty_colmajor(n, k, dtype=torch.float64, device=A.device)
    info = SolveInfo()
    _check(_bind_solver("later_c_spd_solve")(_stream(stream), n, k, A.data_ptr(), _ld(A, "A"), B.data_ptr(),
                                             _ld(B, "B"), X.data_ptr(), _ld(X, "X"), work.data_ptr(), work.numel(),
                                             hwork.data_ptr(), hwork.numel(), ctypes.byref(o), max_iter, tol,
                                             ctypes.byref(info)), "later_c_spd_solve")
    return X, {"iterations": info.iterations, "backward_error": info.backward_error,
               "factor_precision": info.factor_precision}


def ls_solve(A, B, *, precision="split3", max_iter=30, tol=1e-6, work=None, hwork=None, stream=None):
    """Least-squares solve with FP64-residual refinement; returns (X (FP64), info dict)."""
    import torch
    m, n = A.shape
    k = B.shape[1]
    o = Options.make(precision)
    lw, lh = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().later_c_ls_solve_bufsize(m, n, k, ctypes.byref(o), ctypes.byref(lw), ctypes.byref(lh)), "bufsize")
    work, hwork = _solve_ws(lw.value, lh.value, A.device, work, hwork)
    X = empty_colmajor(n, k, dtype=torch.float64, device=A.device)
    info = SolveInfo()
    _check(_bind_solver("later_c_ls_solve")(_stream(stream), m, n, k, A.data_ptr(), _ld(A, "A"), B.data_ptr(),
                                            _ld(B, "B"), X.data_ptr(), _ld(X, "X"), work.data_ptr(), work.numel(),
                                            hwork.data_ptr(), hwork.numel(), ctypes.byref(o), max_iter, tol,
                                            ctypes.byref(info)), "later_c_ls_solve")
    return X, {"iterations": info.iterations, "backward_error": info.backward_error,
               "factor_precision": info.factor_precision}


class BatchedQR:
    """Plan once, run many times (the run is one launch and can be captured in a CUDA graph).

    `mats` are column-major FP32 CUDA tensors (m_i x n_i, m_i >= n_i, n_i <= 256); Q_i overwrites them and
    R_i (n_i x n_i) is written into `rs` (allocated when not given).
    """

    def __init__(self, mats, rs=None, stream=None):
        import torch
        self.mats = list(mats)
        dev = self.mats[0].device
        self.rs = rs if rs is not None else [empty_colmajor(a.shape[1], a.shape[1], device=dev) for a in self.mats]
        items = (QrItem * len(self.mats))()
        for i, (a, r) in enumerate(zip(self.mats, self.rs)):
            items[i] = QrItem(a.data_ptr(), r.data_ptr(), _ld(a, "A"), _ld(r, "R"), a.shape[0], a.shape[1])
        nb = int(lib().later_c_batched_plan_bytes(len(self.mats)))
        self.plan = torch.empty(nb, dtype=torch.uint8, device=dev)
        self.queue = torch.zeros(1, dtype=torch.int32, device=dev)
        self.status = torch.zeros(len(self.mats), dtype=torch.int32, device=dev)
        _check(lib().later_c_batched_qr_plan(_stream(stream), len(self.mats), ctypes.cast(items, ctypes.c_void_p),
                                             self.plan.data_ptr(), nb), "batched_qr_plan")

    def run(self, variant=-1, stream=None):
        _check(lib().later_c_batched_qr_run(_stream(stream), len(self.mats), self.plan.data_ptr(),
                                            self.queue.data_ptr(), self.status.data_ptr(), int(variant)),
               "batched_qr_run")
        return self.rs


class LsServer:
    """Continuous-batching least-squares server (native C++ workers; see later_c.h).

    submit(A, B) takes column-major float32 numpy arrays (host) and returns a ticket;
    wait(ticket) returns (X float64 (n x nrhs), result dict with latency figures).
    """

    def __init__(self, slots=4, hbm_budget_gb=16.0, precision="split3", max_iter=30, tol=1e-6, device=0):
        o = Options.make(precision)
        self._h = lib().later_c_ls_server_create(device, slots, int(hbm_budget_gb * (1 << 30)), ctypes.byref(o),
                                                 max_iter, tol)
        if not self._h:
            raise LaterError(3, "later_c_ls_server_create")
        self._keep = {}

    def submit(self, A, B):
        import numpy as np
        A = np.asfortranarray(A, dtype=np.float32)
        B = np.asfortranarray(B.reshape(B.shape[0], -1), dtype=np.float32)
        m, n = A.shape
        k = B.shape[1]
        X = np.zeros((n, k), dtype=np.float64, order="F")
        req = LsRequest(m, n, k, 0, A.ctypes.data, B.ctypes.data, X.ctypes.data, m, m, n, 0)
        t = lib().later_c_ls_server_submit(self._h, ctypes.byref(req))
        if t < 0:
            raise LaterError(int(-t), "later_c_ls_server_submit")
        self._keep[t] = (A, B, X)
        return t

    def wait(self, ticket):
        res = LsResult()
        _check(lib().later_c_ls_server_wait(self._h, ticket, ctypes.byref(res)), "later_c_ls_server_wait")
        A, B, X = self._keep.pop(ticket)
        return X, res.as_dict()

    def hbm_in_use(self):
        return int(lib().later_c_ls_server_hbm_in_use(self._h))

    def hbm_peak(self):
        return int(lib().later_c_ls_server_hbm_peak(self._h))

    def close(self):
        if self._h:
            lib().later_c_ls_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gemm16(transa, transb, A, B, alpha=1.0, beta=0.0, C=None, D=None, precision="fp16", work=None, stream=None):
    """D = alpha op(A) op(B) + beta C on the tensor cores; A, B 16-bit column-major, C/D FP32."""
    import torch
    ta, tb = transa.upper(), transb.upper()
    m = A.shape[0] if ta == "N" else A.shape[1]
    k = A.shape[1] if ta == "N" else A.shape[0]
    n = B.shape[1] if tb == "N" else B.shape[0]
    if D is None:
        D = empty_colmajor(m, n, device=A.device)
    lda, ldb, ldd = _ld(A, "A"), _ld(B, "B"), _ld(D, "D")
    ldc = _ld(C, "C") if C is not None else m
    wp, wn = (work.data_ptr(), work.numel()) if work is not None else (None, 0)
    _check(lib().later_c_gemm16(_stream(stream), ta.encode(), tb.encode(), m, n, k, alpha, A.data_ptr(), lda,
                                B.data_ptr(), ldb, beta, C.data_ptr() if C is not None else None, ldc,
                                D.data_ptr(), ldd, PREC[precision], wp, wn), "gemm16")
    return D


def convert16(A, precision="fp16", stream=None):
    """FP32 -> 16-bit copy (SPLIT3: returns (hi, lo) with lo = fp16((x - hi) * 2048))."""
    import torch
    m, n = A.shape
    dt = torch.bfloat16 if precision == "bf16" else torch.float16
    ldh = (m + 7) // 8 * 8
    hi = empty_colmajor(m, n, dtype=dt, device=A.device, ld=ldh)
    lo = empty_colmajor(m, n, dtype=dt, device=A.device, ld=ldh) if precision == "split3" else None
    _check(lib().later_c_convert(_stream(stream), m, n, A.data_ptr(), _ld(A, "A"), hi.data_ptr(),
                                 lo.data_ptr() if lo is not None else None, ldh, PREC[precision]), "convert16")
    return (hi, lo) if precision == "split3" else hi

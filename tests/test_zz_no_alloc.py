"""later_c_gemm16_noalloc: the tensor-core GEMM for callers that cannot allocate device memory.

Such callers (a host framework whose memory pool owns the device and forbids
plug-ins from calling the allocator, or a latency-critical path that cannot
afford cudaMalloc's implicit synchronisation) get their split-K scratch from a
fixed array inside the library. This file is collected last so that a run
stopping at the first failure has already run every other test.
"""
import ctypes

import pytest
import torch

import later_gb300 as lg

pytestmark = pytest.mark.gpu

_vp, _i, _f, _c = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_char


def _noalloc():
    fn = lg.lib().later_c_gemm16_noalloc
    fn.restype = _i
    fn.argtypes = [_vp, _c, _c, _i, _i, _i, _f, _vp, _i, _vp, _i, _f, _vp, _i, _vp, _i, _i]
    return fn


def _rel_tol(k):  # the tolerance of tests/test_gemm_gpu.py
    return 1e-6 + 2e-7 * k ** 0.5


def _operand(rows, cols, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    out = lg.empty_colmajor(rows, cols, dtype=torch.float16)
    out.copy_(torch.randn(rows, cols, generator=g, device="cuda"))
    return out


def _call_noalloc(ta, tb, A, B, m, n, k, D):
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return _noalloc()(st, ta.encode(), tb.encode(), m, n, k, 1.0, A.data_ptr(), A.stride(1), B.data_ptr(),
                      B.stride(1), 0.0, None, m, D.data_ptr(), D.stride(1), 0)


@pytest.mark.parametrize("ta,tb,m,n,k", [("T", "N", 256, 256, 16384), ("N", "N", 640, 384, 4096)])
def test_noalloc_matches_gemm16_twice(cuda, ta, tb, m, n, k):
    A = _operand(k if ta == "T" else m, m if ta == "T" else k, 1)
    B = _operand(k, n, 2)
    work = torch.empty(1 << 24, dtype=torch.float32, device="cuda")
    ref = lg.gemm16(ta, tb, A, B, work=work)
    for _ in range(2):  # two calls in a row: the shared array keeps the previous call's contents
        D = lg.empty_colmajor(m, n)
        D.fill_(float("nan"))
        assert _call_noalloc(ta, tb, A, B, m, n, k, D) == 0
        assert lg.device_status() == 0
        err = float((D.double() - ref.double()).norm() / ref.double().norm())
        assert err < _rel_tol(k), err
        # and against the exact product of the same 16-bit operands, in FP64
        a = A.double() if ta == "N" else A.double().t()
        exact = a @ B.double()
        err64 = float((D.double() - exact).norm() / exact.norm())
        assert err64 < _rel_tol(k), err64


@pytest.mark.parametrize("m,n,k", [(4096, 4096, 64), (2048, 4096, 4096)])
def test_noalloc_outputs_beyond_the_array(cuda, m, n, k):
    """Outputs larger than the fixed array (16M and 8M elements against 4M floats) are accepted: they
    fill the SMs with tiles and run without split-K, so the array is not touched. FP64 check."""
    A = _operand(k, m, 3)
    B = _operand(k, n, 4)
    D = lg.empty_colmajor(m, n)
    assert _call_noalloc("T", "N", A, B, m, n, k, D) == 0
    assert lg.device_status() == 0
    exact = A.double().t() @ B.double()
    err64 = float((D.double() - exact).norm() / exact.norm())
    assert err64 < _rel_tol(k), err64

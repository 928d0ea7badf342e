"""Tensor-core GEMM (tcgen05 / TMA / TMEM) against an FP64 product of the same 16-bit operands."""
import pytest
import torch

import later_gb300 as lg

pytestmark = pytest.mark.gpu

# Tolerance: FP32 accumulation of K exact products of 16-bit values; the
# rounding error grows like sqrt(K) u32. A wrong layout / descriptor gives O(1).
def rel_tol(k):
    return 1e-6 + 2e-7 * k ** 0.5


def _ref(ta, tb, A, B, alpha, beta, C):
    a = A.double()
    b = B.double()
    a = a if ta == "N" else a.t()
    b = b if tb == "N" else b.t()
    r = alpha * (a @ b)
    if C is not None and beta != 0:
        r = r + beta * C.double()
    return r


def _operand(rows, cols, dt, ld=None, gen=None):
    x = torch.randn(rows, cols, generator=gen, device="cuda").to(dt)
    out = lg.empty_colmajor(rows, cols, dtype=dt, ld=ld)
    out.copy_(x)
    return out


@pytest.mark.parametrize("ta,tb", [("T", "N"), ("N", "N"), ("N", "T"), ("T", "T")])
@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (256, 256, 256), (200, 136, 72), (384, 64, 1000),
                                   (1024, 512, 512), (64, 64, 4096)])
def test_gemm_layouts(cuda, ta, tb, m, n, k):
    g = torch.Generator(device="cuda").manual_seed(m * 7 + n * 3 + k)
    A = _operand(m if ta == "N" else k, k if ta == "N" else m, torch.float16, gen=g)
    B = _operand(k if tb == "N" else n, n if tb == "N" else k, torch.float16, gen=g)
    D = lg.gemm16(ta, tb, A, B)
    assert lg.device_status() == 0
    ref = _ref(ta, tb, A, B, 1.0, 0.0, None)
    err = (D.double() - ref).norm() / ref.norm()
    assert err < rel_tol(k), float(err)


@pytest.mark.parametrize("prec,dt", [("fp16", torch.float16), ("bf16", torch.bfloat16)])
def test_gemm_alpha_beta_inplace(cuda, prec, dt):
    m, n, k = 640, 384, 320
    g = torch.Generator(device="cuda").manual_seed(5)
    A = _operand(m, k, dt, gen=g)
    B = _operand(k, n, dt, gen=g)
    C = lg.colmajor(torch.randn(m, n, generator=g, device="cuda"))
    ref = _ref("N", "N", A, B, -1.0, 1.0, C)
    lg.gemm16("N", "N", A, B, alpha=-1.0, beta=1.0, C=C, D=C, precision=prec)
    assert lg.device_status() == 0
    err = (C.double() - ref).norm() / ref.norm()
    assert err < rel_tol(k), float(err)


def test_gemm_splitk_deterministic(cuda):
    # Small output, long K: exercises the split-K partial tiles + ticketed reduction.
    m, n, k = 256, 256, 16384
    g = torch.Generator(device="cuda").manual_seed(11)
    A = _operand(k, m, torch.float16, gen=g)
    B = _operand(k, n, torch.float16, gen=g)
    work = torch.empty(1 << 24, dtype=torch.float32, device="cuda")
    D1 = lg.gemm16("T", "N", A, B, work=work)
    D2 = lg.gemm16("T", "N", A, B, work=work)
    assert lg.device_status() == 0
    ref = _ref("T", "N", A, B, 1.0, 0.0, None)
    err = (D1.double() - ref).norm() / ref.norm()
    assert err < rel_tol(k), float(err)
    assert torch.equal(D1, D2)


@pytest.mark.parametrize("m,n,k,beta", [(128, 128, 16384, 0.0), (256, 384, 8192, 1.0), (200, 136, 12000, 1.0),
                                         (1024, 512, 4096, 0.0)])
def test_gemm_splitk_alpha_beta_ragged(cuda, m, n, k, beta):
    """Split-K (partial tiles in `work`, reduced in a fixed order by a second launch) with alpha, beta C and
    ragged tile edges: FP64 check and bit-for-bit repeatable."""
    g = torch.Generator(device="cuda").manual_seed(m + n + k)
    A = _operand(k, m, torch.float16, gen=g)
    B = _operand(k, n, torch.float16, gen=g)
    C = lg.colmajor(torch.randn(m, n, generator=g, device="cuda"))
    work = torch.empty(1 << 24, dtype=torch.float32, device="cuda")
    outs = []
    for _ in range(2):
        outs.append(lg.gemm16("T", "N", A, B, alpha=0.5, beta=beta, C=C if beta else None, work=work))
        assert lg.device_status() == 0
    ref = _ref("T", "N", A, B, 0.5, beta, C)
    err = (outs[0].double() - ref).norm() / ref.norm()
    assert err < rel_tol(k), float(err)
    assert torch.equal(outs[0], outs[1])


def test_gemm_leading_dims(cuda):
    m, n, k = 300, 200, 136
    g = torch.Generator(device="cuda").manual_seed(3)
    A = _operand(k, m, torch.float16, ld=k + 24, gen=g)
    B = _operand(k, n, torch.float16, ld=k + 8, gen=g)
    D = lg.empty_colmajor(m, n, ld=m + 5)
    lg.gemm16("T", "N", A, B, D=D)
    ref = _ref("T", "N", A, B, 1.0, 0.0, None)
    assert (D.double() - ref).norm() / ref.norm() < rel_tol(k)


# The shapes below make tc_gemm pick BN = 256 (tiles_m * ceil(N / 256) >= the SM count) with no split-K,
# so they run the persistent kernels that carry the 16384^2 QR: the top-level projection R12 = Q1^T A2 (TN)
# and the update A2 -= Q1 R12 (NN, in place, alpha = -1, beta = 1).
@pytest.mark.parametrize("prec,dt", [("fp16", torch.float16), ("bf16", torch.bfloat16)])
def test_gemm_persistent_bn256_projection(cuda, prec, dt):
    m, n, k = 4096, 4096, 8192
    g = torch.Generator(device="cuda").manual_seed(41)
    A = _operand(k, m, dt, gen=g)
    B = _operand(k, n, dt, gen=g)
    work = torch.empty(1 << 24, dtype=torch.float32, device="cuda")
    D = lg.gemm16("T", "N", A, B, precision=prec, work=work)
    assert lg.device_status() == 0
    ref = _ref("T", "N", A, B, 1.0, 0.0, None)
    err = (D.double() - ref).norm() / ref.norm()
    assert err < rel_tol(k), float(err)


def test_gemm_persistent_bn256_update(cuda):
    m, n, k = 16384, 2048, 2048
    g = torch.Generator(device="cuda").manual_seed(43)
    A = _operand(m, k, torch.float16, gen=g)
    B = _operand(k, n, torch.float16, gen=g)
    C = lg.colmajor(torch.randn(m, n, generator=g, device="cuda"))
    ref = _ref("N", "N", A, B, -1.0, 1.0, C)
    work = torch.empty(1 << 24, dtype=torch.float32, device="cuda")
    lg.gemm16("N", "N", A, B, alpha=-1.0, beta=1.0, C=C, D=C, work=work)
    assert lg.device_status() == 0
    err = (C.double() - ref).norm() / ref.norm()
    assert err < rel_tol(k), float(err)

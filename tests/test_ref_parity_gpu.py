"""Parity against the reference LATER itself, run on this GPU (oracle/_ref): its own MGS panel and
conversion kernels compiled from its sources, its host recursion restated call for call around them and
the same cuBLAS / cuSOLVER calls. Two things are checked on the same seeded inputs:

1. the oracle's restatement reproduces the reference's outputs (this is what pins the oracle);
2. this library's results meet the reference's own error levels (north-star: "results must match the
   reference's own rgsqrf / rpotrf error bounds on the same seeded inputs").
"""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen, metrics
from oracle import later_oracle as lo
from tests.gpu_metrics import qr_errors_fp64

pytestmark = pytest.mark.gpu


def _dev(A):
    return lg.colmajor(torch.from_numpy(np.ascontiguousarray(A)).cuda())


def ref_rgsqrf(ref, A):
    m, n = A.shape
    dA = _dev(A) if isinstance(A, np.ndarray) else A
    R = torch.zeros(n, n, device="cuda").t()
    lw, lh = ref.rgsqrf_bufsize(m, n)
    work = torch.zeros(max(lw, m // 256 * 32 * 64), device="cuda")
    hwork = torch.zeros(lh, dtype=torch.float16, device="cuda")
    ref.rgsqrf(dA, R, work, hwork)
    torch.cuda.synchronize()
    return dA, torch.triu(R)


@pytest.mark.parametrize("m", [512, 4096, 16384])
def test_oracle_leaf_reproduces_reference_panels(ref, m):
    """n = 128: one mgs_caqr_panel_256x128 (the reference's mgs_kernel2 TSQR trees and FP32 Sgemm
    glue). The oracle's restatement agrees with it to FP32 rounding, entry by entry."""
    A = gen.normal(m, 128, seed=m + 1)
    dQ, dR = ref_rgsqrf(ref, A)
    Q, R = dQ.cpu().numpy(), dR.cpu().numpy()
    Qo, Ro = lo.rgsqrf(A)
    assert np.abs(Q - Qo).max() <= 2e-5 * np.abs(Qo).max(), np.abs(Q - Qo).max()
    assert np.abs(R - np.triu(Ro)).max() <= 2e-5 * np.abs(Ro).max()


@pytest.mark.parametrize("m,n", [(1024, 256), (4096, 1024)])
def test_oracle_rgsqrf_reproduces_reference(ref, m, n):
    """The whole recursion in the reference's FP16 arithmetic: the oracle's Q and R match the
    reference's to the size of one FP16 rounding of an operand, and their FP64 errors agree."""
    A = gen.normal(m, n, seed=m + n)
    dQ, dR = ref_rgsqrf(ref, A)
    Q, R = dQ.cpu().numpy(), dR.cpu().numpy()
    Qo, Ro = lo.rgsqrf(A, prec="fp16")
    assert np.linalg.norm(Q - Qo) / np.linalg.norm(Qo) <= 2e-3
    assert np.linalg.norm(R - np.triu(Ro)) / np.linalg.norm(Ro) <= 2e-3
    b, bo = metrics.qr_backward_error(A, Q, R), metrics.qr_backward_error(A, Qo, Ro)
    o, oo = metrics.orthogonality(Q), metrics.orthogonality(Qo)
    assert 0.5 * bo <= b <= 2.0 * bo, (b, bo)
    assert 0.5 * oo <= o <= 2.0 * oo + 1e-6, (o, oo)


@pytest.mark.parametrize("m,n,kappa", [(4096, 1024, None), (4096, 1024, 1e3), (4096, 1024, 1e5),
                                       (16384, 2048, None)])
def test_rgsqrf_meets_reference_error_levels(ref, m, n, kappa):
    """This library's rgsqrf on the reference's own inputs: in FP16 (the reference's only mode) the
    backward error and orthogonality are within 2x of the reference's; SPLIT2 is at least 10x better."""
    A = gen.normal(m, n, seed=3 * m + n) if kappa is None else gen.svd_matrix(m, n, kappa, seed=int(kappa))
    dQr, dRr = ref_rgsqrf(ref, A)
    A0 = _dev(A)
    b_ref, o_ref = qr_errors_fp64(A0, dQr, dRr)
    out = {}
    for prec in ("fp16", "split2"):
        dA = _dev(A)
        R = lg.later_rgsqrf(dA, precision=prec)
        assert lg.device_status() == 0
        out[prec] = qr_errors_fp64(A0, dA, R)
    assert out["fp16"][0] <= 2.0 * b_ref, (out["fp16"], b_ref)
    assert out["fp16"][1] <= 2.0 * o_ref + 1e-6, (out["fp16"], o_ref)
    assert out["split2"][0] <= 0.1 * b_ref, (out["split2"], b_ref)


def test_rgsqrf_meets_reference_at_headline_size(ref):
    """16384^2, the benchmark's matrix (N(0,1), seed 1 on the device): the reference in FP16 and this
    library in SPLIT2 (the benchmark's headline mode) and FP16, FP64 errors."""
    m = n = 16384
    g = torch.Generator(device="cuda").manual_seed(1)
    A0 = torch.randn(n, m, generator=g, device="cuda").t()
    A = lg.empty_colmajor(m, n)
    A.copy_(A0)
    Qr, Rr = ref_rgsqrf(ref, A)
    b_ref, o_ref = qr_errors_fp64(A0, Qr, Rr)
    del Qr, Rr
    for prec, fac in (("fp16", 2.0), ("split2", 0.1)):
        A = lg.empty_colmajor(m, n)
        A.copy_(A0)
        R = lg.later_rgsqrf(A, precision=prec)
        assert lg.device_status() == 0
        b, o = qr_errors_fp64(A0, A, R)
        assert b <= fac * b_ref, (prec, b, b_ref)
        assert o <= 2.0 * o_ref + 1e-6, (prec, o, o_ref)
        del A, R
    assert b_ref > 1e-5  # the reference's FP16 arithmetic does not reach the 1e-5 target; SPLIT2 does


def test_rpotrf_meets_reference_error_level(ref):
    """n = 4096 SPD (kappa 1e2): the reference's l_potrf (cuSOLVER Spotrf leaves of 2048, its
    recursive trsm / syrk with FP16 GemmEx) against this library's rpotrf, FP64 backward errors; the
    oracle's restatement sits at the reference's level."""
    n = 4096
    A = gen.spd_matrix(n, 1e2, seed=12)
    dA = _dev(A)
    hwork = torch.zeros(n // 2 * n, dtype=torch.float16, device="cuda")
    info = ref.rpotrf(dA, hwork)
    assert info == 0
    L_ref = np.tril(dA.cpu().numpy())
    b_ref = metrics.chol_backward_error(A, L_ref)
    dB = _dev(A)
    lg.later_rpotrf("l", n, dB)
    assert lg.device_status() == 0
    b = metrics.chol_backward_error(A, np.tril(dB.cpu().numpy()))
    b_or = metrics.chol_backward_error(A, lo.rpotrf(A))
    assert b <= 2.0 * b_ref, (b, b_ref)
    assert 0.33 * b_ref <= b_or <= 3.0 * b_ref, (b_or, b_ref)

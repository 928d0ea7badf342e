"""Pins the CPU oracle (the numpy restatement of the reference's algorithms).

The reference ships no golden vectors, so the restatement is pinned by
mathematics the reference's outputs must satisfy: the thin QR with a positive
diagonal is unique (rgsqrf, MGS R_kk > 0, QR/panel.cu:281-284), and the
Householder reconstruction with the sign choice must reproduce LAPACK dgeqrf's
reflectors and R (rhouqr). Also checks the committed fixtures in tests/golden/.
"""
import numpy as np
import pytest

from oracle import gen, metrics
from oracle import later_oracle as lo


@pytest.mark.parametrize("m,n", [(256, 32), (1000, 64), (3000, 256)])
def test_rgsqrf_oracle_matches_lapack_fp32_levels(m, n):
    # With split3 (~FP32) trailing updates the oracle must equal LAPACK's unique QR.
    A = gen.normal(m, n, seed=m)
    Q, R = lo.rgsqrf(A, prec="split3")
    Qx, Rx = metrics.lapack_qr_positive(A)
    assert np.linalg.norm(R - Rx) / np.linalg.norm(Rx) < 2e-6
    assert np.linalg.norm(Q - Qx) / np.linalg.norm(Qx) < 2e-5


def test_rgsqrf_oracle_fp16_error_model():
    # FP16 trailing updates: backward error at the FP16 product level (~1e-4), not worse.
    A = gen.normal(2048, 512, seed=1)
    Q, R = lo.rgsqrf(A, prec="fp16")
    e = metrics.qr_backward_error(A, Q, R)
    assert 1e-5 < e < 5e-4


def test_rgsqrf_oracle_split2_error_model():
    # split2: the subtracted R12 is the stored one and Q1 enters the update as hi + lo, so the
    # backward error drops to the FP32 level while orthogonality stays at the FP16 level.
    A = gen.normal(2048, 512, seed=1)
    Q2, R2 = lo.rgsqrf(A, prec="split2")
    Qh, Rh = lo.rgsqrf(A, prec="fp16")
    assert metrics.qr_backward_error(A, Q2, R2) < 1e-6
    assert metrics.orthogonality(Q2) < 2 * metrics.orthogonality(Qh) + 1e-6


def test_mgs_block_and_tsqr_agree():
    A = gen.normal(2000, 32, seed=5)
    q1, r1 = lo.mgs_block(A)
    q2, r2 = lo.tsqr32(A)
    assert np.allclose(r1, r2, rtol=1e-4, atol=1e-4)
    assert np.allclose(q1, q2, atol=1e-5)


def test_mgs_block_rank_deficient_rows():
    A = gen.normal(10, 32, seed=2)  # fewer rows than columns
    q, r = lo.mgs_block(A)
    assert np.all(q[:, 10:] == 0) and np.all(r[10:, 10:] == 0)
    assert np.allclose(q @ r, A, atol=1e-4)


@pytest.mark.parametrize("m,n", [(512, 32), (1000, 96), (700, 64)])
def test_rhouqr_oracle_matches_lapack(m, n):
    import scipy.linalg.lapack as la
    A = gen.normal(m, n, seed=n)
    Y, W, R = lo.rhouqr(A)
    qr, tau, _, _ = la.dgeqrf(A.astype(np.float64))
    V = np.tril(qr, -1) + np.eye(m, n)
    assert np.linalg.norm(Y - V) / np.linalg.norm(V) < 1e-5
    assert np.linalg.norm(np.triu(R) - np.triu(qr[:n])) / np.linalg.norm(np.triu(qr[:n])) < 1e-5
    Q = lo.ormqr(W, Y)
    assert metrics.qr_backward_error(A, Q, R) < 1e-6
    assert metrics.orthogonality(Q) < 1e-5


def test_reconstruction_is_sign_invariant():
    # Flipping column signs of the input Q (and rows of R) must not change (Y, T, R').
    A = gen.normal(300, 32, seed=3)
    q, r = lo.tsqr32(A)
    d = np.where(np.arange(32) % 3 == 0, -1.0, 1.0).astype(np.float32)
    y1, w1, r1, t1 = lo.householder_reconstruct(q, r)
    y2, w2, r2, t2 = lo.householder_reconstruct(q * d, d[:, None] * r)
    assert np.allclose(y1, y2, atol=1e-5) and np.allclose(r1, r2, atol=1e-4) and np.allclose(t1, t2, atol=1e-4)


def test_reference_literal_reconstruction_same_product():
    # The reference's S = I variant gives the same A = Q R (R rows may flip sign).
    A = gen.normal(512, 64, seed=8)
    Ys, Ws, Rs = lo.rhouqr(A, signs=True)
    Yi, Wi, Ri = lo.rhouqr(A, signs=False)
    Qs, Qi = lo.ormqr(Ws, Ys), lo.ormqr(Wi, Yi)
    assert np.allclose(Qs @ np.triu(Rs), Qi @ np.triu(Ri), atol=1e-4)
    assert np.allclose(np.abs(np.triu(Rs)), np.abs(np.triu(Ri)), atol=1e-3)

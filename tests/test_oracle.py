"""Pins the CPU oracle (the numpy restatement of the reference's algorithms).

The reference ships no golden vectors. Besides the golden vectors generated
from the reference itself on a GPU (tests/test_golden.py), the restatement is
pinned here by mathematics the reference's outputs must satisfy: the thin QR
with a positive diagonal is unique (rgsqrf, MGS R_kk > 0, QR/panel.cu:281-284),
and the Householder reconstruction with the sign choice must reproduce LAPACK
dgeqrf's reflectors and R (rhouqr).
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


# Known answers on the reference tests' constant inputs (T = lower triangle of 0.1,
# test/test_trsm.cu:44-56, test/test_trmm.cu:43-55, test/test_potrf.cu:38-62): the BLAS-3 and
# Cholesky restatements are pinned to exact results, through their recursion (small leaves).
def _T(n):
    return gen.lower_tri_const(n)


@pytest.mark.parametrize("prec,tol", [("fp16", 6e-4), ("split3", 2e-6)])
def test_rtrmm_oracle_known_answer(prec, tol):
    n = 512
    C = lo.rtrmm(_T(n), np.ones((n, 48), np.float32), prec=prec, leaf=64)
    exact = np.repeat(0.1 * np.arange(1, n + 1, dtype=np.float64)[:, None], 48, axis=1)
    assert np.abs(C - exact).max() / np.abs(exact).max() < tol


@pytest.mark.parametrize("prec,tol", [("fp16", 1e-3), ("split3", 2e-6)])
def test_rsyrk_oracle_known_answer(prec, tol):
    n = 384
    C = lo.rsyrk(1.0, _T(n), 0.0, np.zeros((n, n), np.float32), prec=prec)
    i = np.arange(n)
    exact = 0.01 * (np.minimum.outer(i, i) + 1)
    il = np.tril_indices(n)
    assert np.abs(C[il] - exact[il]).max() / exact.max() < tol
    assert np.all(np.triu(C, 1) == 0)  # the upper triangle is not touched


@pytest.mark.parametrize("side", ["l", "r"])
def test_rtrsm_oracle_known_answer(side):
    n, k = 512, 40
    T = _T(n).astype(np.float64)
    B = (T @ np.ones((n, k))) if side == "l" else (np.ones((k, n)) @ T.T)
    B = B.astype(np.float32)
    X3 = lo.rtrsm(side, _T(n), B, prec="split3", leaf=64)
    assert np.abs(X3 - 1.0).max() < 1e-3  # the exact answer is all ones
    X16 = lo.rtrsm(side, _T(n), B, prec="fp16", leaf=64).astype(np.float64)
    res = (T @ X16 - B) if side == "l" else (X16 @ T.T - B)
    assert np.linalg.norm(res) / np.linalg.norm(B) < 1e-3


def test_rpotrf_oracle_known_answer():
    n = 512
    T = _T(n).astype(np.float64)
    A = (T @ T.T).astype(np.float32)
    L3 = lo.rpotrf(A, prec="split3", leaf=128).astype(np.float64)
    assert np.linalg.norm(L3 - T) / np.linalg.norm(T) < 1e-3  # the factor of T T^T is T
    L16 = lo.rpotrf(A, prec="fp16", leaf=128).astype(np.float64)
    assert metrics.chol_backward_error(A, L16) < 1e-3


@pytest.mark.parametrize("m,n", [(1000, 256), (700, 384)])
def test_oracle_bhouqr_is_lapack_householder_form(m, n):
    """later_bhouqr's restatement (FP32, the reference's arithmetic) gives LAPACK dgeqrf's reflectors and R,
    and Q = I - W Y^T (the reference's later_ormqr2) is orthonormal with A = Q R."""
    import scipy.linalg.lapack as la
    A = gen.normal(m, n, seed=3)
    Y, W, R = lo.bhouqr(A)
    Q = lo.ormqr(W, Y)
    qr, tau, _, _ = la.dgeqrf(A.astype(np.float64))
    Rl = np.triu(qr[:n])
    V = np.tril(qr, -1) + np.eye(m, n)
    assert np.linalg.norm(R - Rl) / np.linalg.norm(Rl) < 2e-6
    assert np.linalg.norm(Y - V) / np.linalg.norm(V) < 2e-6
    assert metrics.qr_backward_error(A, Q, R) < 2e-6
    assert metrics.orthogonality(Q) < 1e-4

"""FP64 accuracy metrics (host LAPACK via numpy / scipy).

The reference prints the same quantities computed in FP32 with cuBLAS
(test/test_qr.cu:216-228 backward error, :245-268 orthogonality divided by n);
here they are computed in FP64 on the host.
"""
from __future__ import annotations

import numpy as np


def qr_backward_error(A, Q, R) -> float:
    """||A - Q R||_F / ||A||_F in FP64."""
    A = np.asarray(A, dtype=np.float64)
    Q = np.asarray(Q, dtype=np.float64)
    R = np.triu(np.asarray(R, dtype=np.float64))
    return float(np.linalg.norm(A - Q @ R) / np.linalg.norm(A))


def orthogonality(Q) -> float:
    """||I - Q^T Q||_F in FP64 (the reference additionally divides by n)."""
    Q = np.asarray(Q, dtype=np.float64)
    n = Q.shape[1]
    return float(np.linalg.norm(np.eye(n) - Q.T @ Q))


def lapack_qr_positive(A):
    """FP64 LAPACK QR (dgeqrf/dorgqr) with R's diagonal made positive.

    With a positive diagonal the thin QR of a full-rank matrix is unique, so
    this is the exact factor rgsqrf approximates (MGS gives R_kk = ||a_k|| > 0,
    QR/panel.cu:281-284).
    """
    q, r = np.linalg.qr(np.asarray(A, dtype=np.float64))
    s = np.sign(np.diag(r))
    s[s == 0] = 1.0
    return q * s[None, :], r * s[:, None]


def chol_backward_error(A, L) -> float:
    """||A - L L^T||_F / ||A||_F in FP64 (test/test_potrf.cu:92)."""
    A = np.asarray(A, dtype=np.float64)
    L = np.tril(np.asarray(L, dtype=np.float64))
    return float(np.linalg.norm(A - L @ L.T) / np.linalg.norm(A))


def solve_backward_error(A, x, b) -> float:
    """Normwise backward error ||b - A x|| / (||A|| ||x|| + ||b||), FP64, per column max."""
    A = np.asarray(A, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if x.ndim == 1:
        x, b = x[:, None], b[:, None]
    r = b - A @ x
    na = np.linalg.norm(A, 2) if min(A.shape) <= 2048 else np.linalg.norm(A)
    e = np.linalg.norm(r, axis=0) / (na * np.linalg.norm(x, axis=0) + np.linalg.norm(b, axis=0))
    return float(e.max())

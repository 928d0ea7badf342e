"""Seeded synthetic inputs with the shapes and distributions of the benchmark configs.

The reference generates its test inputs on the GPU with cuRAND (U(0,1), fixed
seed 3000; util/util.cu:102-109); here every input is produced by numpy's
PCG64 generator from an explicit seed so the same matrix can be rebuilt on any
machine.
"""
from __future__ import annotations

import numpy as np


def normal(m: int, n: int, seed: int, dtype=np.float32) -> np.ndarray:
    """i.i.d. N(0,1), column-major (Fortran order)."""
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.standard_normal((m, n), dtype=np.float64).astype(dtype))


def uniform(m: int, n: int, seed: int, dtype=np.float32) -> np.ndarray:
    """i.i.d. U(0,1) — the distribution of the reference's generateUniformMatrix."""
    rng = np.random.default_rng(seed)
    return np.asfortranarray(rng.random((m, n)).astype(dtype))


def haar(n: int, k: int, rng: np.random.Generator) -> np.ndarray:
    """n x k matrix with Haar-distributed orthonormal columns (FP64).

    QR of a Gaussian matrix with the signs of R's diagonal moved into Q
    (Mezzadri, "How to generate random matrices from the classical compact
    groups", Notices AMS 54, 2007).
    """
    g = rng.standard_normal((n, k))
    q, r = np.linalg.qr(g)
    return q * np.sign(np.diag(r))[None, :]


def svd_matrix(m: int, n: int, kappa: float, seed: int, dtype=np.float32) -> np.ndarray:
    """A = U diag(sigma) V^T, U / V Haar, sigma geometric from 1 to 1/kappa."""
    rng = np.random.default_rng(seed)
    u = haar(m, n, rng)
    v = haar(n, n, rng)
    sig = np.geomspace(1.0, 1.0 / kappa, n)
    return np.asfortranarray(((u * sig[None, :]) @ v.T).astype(dtype))


def spd_matrix(n: int, kappa: float, seed: int, dtype=np.float32) -> np.ndarray:
    """A = Q diag(lambda) Q^T, Q Haar, lambda log-uniform in [1/kappa, 1]."""
    rng = np.random.default_rng(seed)
    q = haar(n, n, rng)
    lam = np.exp(rng.uniform(np.log(1.0 / kappa), 0.0, n))
    a = (q * lam[None, :]) @ q.T
    a = 0.5 * (a + a.T)
    return np.asfortranarray(a.astype(dtype))


def lower_tri_const(n: int, v: float = 0.1, dtype=np.float32) -> np.ndarray:
    """Lower triangle (with diagonal) filled with v — the reference tests' L
    (test/test_trsm.cu:44-49, test/test_trmm.cu:43-48, test/test_potrf.cu:38-46)."""
    return np.asfortranarray(np.tril(np.full((n, n), v, dtype=dtype)))

"""later_sy2sb on the GPU (EVD/later_sy2sb_blocked.cu:23-186, EVD/later_sy2sb_rec.cu): symmetric to band
reduction B = Q^T A Q over rhouqr panels and two-sided ZY tensor-core updates. Checked in FP64: the band
structure is exact, the eigenvalues are preserved, Q^T A Q = B with Q rebuilt from the returned
reflectors, and the result agrees with the oracle's restatement."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen
from oracle import later_oracle as lo

pytestmark = pytest.mark.gpu


def _sym(n, seed, kappa=None):
    rng = np.random.default_rng(seed)
    q = gen.haar(n, n, rng)
    lam = rng.standard_normal(n) if kappa is None else np.geomspace(1.0, 1.0 / kappa, n) * rng.choice([-1, 1], n)
    A = (q * lam[None, :]) @ q.T
    return ((A + A.T) / 2).astype(np.float32)


def _q_from(Y, W, n, nb):
    Q = np.eye(n)
    for i in range(0, n - nb, nb):
        Q = Q @ (np.eye(n) - W[:, i:i + nb].astype(np.float64) @ Y[:, i:i + nb].T.astype(np.float64))
    return Q


@pytest.mark.parametrize("n,nb,prec,tol", [(512, 64, "split3", 2e-6), (1024, 128, "split3", 2e-6),
                                           (768, 32, "split3", 2e-6), (1024, 128, "fp16", 2e-3),
                                           (2048, 128, "split3", 3e-6)])
def test_sy2sb_band_eigenvalues_and_similarity(cuda, n, nb, prec, tol):
    A = _sym(n, seed=n + nb)
    dA = lg.colmajor(torch.from_numpy(A).cuda())
    Y, W = lg.later_sy2sb(dA, nb, precision=prec)
    assert lg.device_status() == 0
    B = dA.cpu().numpy()
    assert np.all(np.triu(B, nb + 1) == 0) and np.all(np.tril(B, -nb - 1) == 0)
    # symmetric to rounding: entry (i, j) and (j, i) take the two rank-nb products in opposite order
    assert np.abs(B - B.T).max() <= 10 * tol * np.abs(A).max()
    ev = np.linalg.eigvalsh(B.astype(np.float64))
    ev0 = np.linalg.eigvalsh(A.astype(np.float64))
    assert np.abs(ev - ev0).max() <= tol * np.abs(ev0).max(), np.abs(ev - ev0).max()
    Q = _q_from(Y.cpu().numpy(), W.cpu().numpy(), n, nb)
    assert np.linalg.norm(Q.T @ A.astype(np.float64) @ Q - B) / np.linalg.norm(A) <= 50 * tol
    if n <= 1024:
        Bo, _, _ = lo.sy2sb(A, nb=nb, prec=prec)
        evo = np.linalg.eigvalsh(Bo.astype(np.float64))
        assert np.abs(ev - ev0).max() <= 3 * np.abs(evo - ev0).max() + 1e-6 * np.abs(ev0).max()


def test_sy2sb_ill_conditioned_spectrum(cuda):
    n, nb = 1024, 128
    A = _sym(n, seed=9, kappa=1e5)
    dA = lg.colmajor(torch.from_numpy(A).cuda())
    lg.later_sy2sb(dA, nb, reflectors=False)
    assert lg.device_status() == 0
    B = dA.cpu().numpy()
    ev = np.linalg.eigvalsh(B.astype(np.float64))
    ev0 = np.linalg.eigvalsh(A.astype(np.float64))
    assert np.abs(ev - ev0).max() <= 3e-6

"""later_bhouqr / later_ormqr2 on the GPU: blocked Householder QR over 128-column rhouqr panels
(QR/later_bhouqr.cu:88-189), against the oracle's restatement and LAPACK dgeqrf's Householder form."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen, metrics
from oracle import later_oracle as lo

pytestmark = pytest.mark.gpu

BOUND = {"fp16": 1e-3, "bf16": 8e-3, "split3": 3e-6}


@pytest.mark.parametrize("m,n,prec", [(256, 128, "split3"), (1000, 256, "split3"), (2048, 512, "split3"),
                                      (4096, 1024, "split3"), (3000, 640, "fp16"), (2048, 384, "bf16"),
                                      (8192, 2048, "split3")])
def test_bhouqr_matches_oracle_and_lapack(cuda, m, n, prec):
    import scipy.linalg.lapack as la
    A = gen.normal(m, n, seed=m + 5 * n)
    dA = lg.colmajor(torch.from_numpy(A).cuda())
    W, R = lg.later_bhouqr(dA, precision=prec)
    assert lg.device_status() == 0
    Y, Wc, Rc = dA.cpu().numpy(), W.cpu().numpy(), R.cpu().numpy()
    lg.later_ormqr2(W, dA)
    assert lg.device_status() == 0
    Q = W.cpu().numpy()
    Yo, Wo, Ro = lo.bhouqr(A, prec=prec)
    Qo = lo.ormqr(Wo, Yo)
    bwd, orth = metrics.qr_backward_error(A, Q, Rc), metrics.orthogonality(Q)
    bwd_o, orth_o = metrics.qr_backward_error(A, Qo, Ro), metrics.orthogonality(Qo)
    assert bwd <= max(3 * bwd_o, 1e-6) and bwd <= BOUND[prec], (bwd, bwd_o)
    assert orth <= max(3 * orth_o, 2e-5), (orth, orth_o)
    assert np.all(np.tril(Rc, -1) == 0)
    assert np.allclose(np.diag(Y[:n]), 1.0) and np.all(np.triu(Y[:n], 1) == 0)
    qr, tau, _, _ = la.dgeqrf(A.astype(np.float64))
    Rl = np.triu(qr[:n])
    V = np.tril(qr, -1) + np.eye(m, n)
    tol = max(10 * BOUND[prec], 1e-5)
    assert np.linalg.norm(Rc - Rl) / np.linalg.norm(Rl) < tol
    assert np.linalg.norm(Y - V) / np.linalg.norm(V) < tol
    assert np.linalg.norm(Wc - Wo) / np.linalg.norm(Wo) < tol


def test_bhouqr_leading_dimensions(cuda):
    m, n = 1500, 256
    A = gen.normal(m, n, seed=8)
    dA = lg.empty_colmajor(m, n, ld=m + 40)
    dA.copy_(torch.from_numpy(A).cuda())
    W = lg.empty_colmajor(m, n, ld=m + 24)
    R = lg.empty_colmajor(n, n, ld=n + 8)
    lg.later_bhouqr(dA, W, R)
    assert lg.device_status() == 0
    lg.later_ormqr2(W, dA)
    assert lg.device_status() == 0
    assert metrics.qr_backward_error(A, W.cpu().numpy(), R.cpu().numpy()) < 3e-6

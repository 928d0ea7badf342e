"""later_rhouqr / later_ormqr on the GPU against the oracle and FP64 LAPACK dgeqrf."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen, metrics
from oracle import later_oracle as lo

pytestmark = pytest.mark.gpu

BOUND = {"fp16": 5e-4, "bf16": 4e-3, "split3": 2e-6}


def run(A, precision="fp16"):
    dA = lg.colmajor(torch.from_numpy(np.ascontiguousarray(A)).cuda())
    W, R = lg.later_rhouqr(dA, precision=precision)
    assert lg.device_status() == 0
    Y, Wc, Rc = dA.cpu().numpy(), W.cpu().numpy(), R.cpu().numpy()
    lg.later_ormqr(W, dA)
    assert lg.device_status() == 0
    return Y, Wc, Rc, W.cpu().numpy()


@pytest.mark.parametrize("m,n,prec", [(256, 32, "fp16"), (512, 64, "fp16"), (1000, 96, "fp16"),
                                      (2048, 512, "fp16"), (4096, 1024, "fp16"), (2048, 512, "split3"),
                                      (3001, 320, "bf16"), (20000, 64, "fp16")])
def test_rhouqr_matches_oracle_and_lapack(cuda, m, n, prec):
    import scipy.linalg.lapack as la
    A = gen.normal(m, n, seed=m + 3 * n)
    Y, W, R, Q = run(A, prec)
    Yo, Wo, Ro = lo.rhouqr(A, prec=prec)
    bwd, orth = metrics.qr_backward_error(A, Q, R), metrics.orthogonality(Q)
    Qo = lo.ormqr(Wo, Yo)
    bwd_o, orth_o = metrics.qr_backward_error(A, Qo, Ro), metrics.orthogonality(Qo)
    assert bwd <= max(3 * bwd_o, 1e-6) and bwd <= BOUND[prec], (bwd, bwd_o)
    assert orth <= max(3 * orth_o, 2e-5), (orth, orth_o)
    # R zero below the diagonal; Y unit lower trapezoidal; same signs as LAPACK.
    assert np.all(np.tril(R, -1) == 0)
    assert np.allclose(np.diag(Y[:n]), 1.0) and np.all(np.triu(Y[:n], 1) == 0)
    qr, tau, _, _ = la.dgeqrf(A.astype(np.float64))
    Rl = np.triu(qr[:n])
    V = np.tril(qr, -1) + np.eye(m, n)
    tol = max(10 * BOUND[prec], 1e-5)
    assert np.linalg.norm(R - Rl) / np.linalg.norm(Rl) < tol
    assert np.linalg.norm(Y - V) / np.linalg.norm(V) < tol
    assert np.linalg.norm(W - Wo) / np.linalg.norm(Wo) < tol


def test_rhouqr_reference_uniform_input(cuda):
    A = gen.uniform(1024, 256, seed=3000)  # the reference test's U(0,1) input
    Y, W, R, Q = run(A)
    assert metrics.qr_backward_error(A, Q, R) < 2e-4
    assert metrics.orthogonality(Q) < 1e-2

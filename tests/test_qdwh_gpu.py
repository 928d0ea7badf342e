"""later_qdwh_polar on the GPU (EVD/later_qdwh_polar.cu:24-110): the polar decomposition A = U H by the
QR-based QDWH iteration over later_rgsqrf, against FP64 LAPACK (scipy.linalg.polar) and the oracle."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen
from oracle import later_oracle as lo

pytestmark = pytest.mark.gpu


def _dev(A):
    return lg.colmajor(torch.from_numpy(np.ascontiguousarray(A)).cuda())


def _check(A, U, H, kappa, orth_tol, bwd_tol):
    import scipy.linalg as sl
    A64 = A.astype(np.float64)
    U64, H64 = U.astype(np.float64), H.astype(np.float64)
    n = A.shape[1]
    orth = np.linalg.norm(U64.T @ U64 - np.eye(n))
    bwd = np.linalg.norm(A64 - U64 @ H64) / np.linalg.norm(A64)
    assert orth <= orth_tol, orth
    assert bwd <= bwd_tol, bwd
    assert np.allclose(H, H.T)
    assert np.linalg.eigvalsh(H64).min() >= -1e-4 * np.linalg.norm(H64, 2)
    Ue, He = sl.polar(A64)
    # the polar factor's sensitivity grows with the condition number
    assert np.linalg.norm(U64 - Ue) / np.linalg.norm(Ue) <= max(5e-5, 50 * kappa * 6e-8)
    return orth, bwd


@pytest.mark.parametrize("m,n,kappa", [(512, 512, 1e1), (1024, 1024, 1e3), (1024, 1024, 1e5), (2048, 512, 1e3),
                                       (4096, 1024, 1e2)])
def test_qdwh_polar_matches_lapack_and_oracle(cuda, m, n, kappa):
    A = gen.svd_matrix(m, n, kappa, seed=m + n)
    U, H, it = lg.later_qdwh_polar(_dev(A))
    assert lg.device_status() == 0
    assert 1 <= it <= 6, it
    orth, bwd = _check(A, U.cpu().numpy(), H.cpu().numpy(), kappa, 1e-4, 1e-5)
    if m * n <= 1024 * 1024:
        Uo, Ho, it_o = lo.qdwh_polar(A)
        orth_o = np.linalg.norm(Uo.T.astype(np.float64) @ Uo - np.eye(n))
        assert orth <= 3 * orth_o + 1e-6, (orth, orth_o)
        assert abs(it - it_o) <= 1, (it, it_o)


def test_qdwh_symmetric_input_like_the_reference(cuda):
    """The reference symmetrises every iterate (its QDWH serves the symmetric eigenproblem)."""
    n = 1024
    rng = np.random.default_rng(5)
    q = gen.haar(n, n, rng)
    lam = np.exp(rng.uniform(np.log(1e-3), 0.0, n)) * rng.choice([-1.0, 1.0], n)  # symmetric, indefinite
    A = (q * lam[None, :]) @ q.T
    A = ((A + A.T) / 2).astype(np.float32)
    U, H, it = lg.later_qdwh_polar(_dev(A), symmetric=True)
    assert lg.device_status() == 0
    Uc = U.cpu().numpy()
    assert np.abs(Uc - Uc.T).max() == 0.0
    _check(A, Uc, H.cpu().numpy(), 1e3, 1e-4, 1e-5)


def test_qdwh_reference_fp16_arithmetic_stalls(cuda):
    """With the reference's plain FP16 products the iterate is only FP16-orthogonal; SPLIT3 (the default)
    reaches the FP32 level on the same input."""
    A = gen.svd_matrix(1024, 1024, 1e2, seed=2)
    U16, _, _ = lg.later_qdwh_polar(_dev(A), precision="fp16", tol=2e-4)
    U32, _, _ = lg.later_qdwh_polar(_dev(A))
    assert lg.device_status() == 0

    def orth(U):
        U = U.cpu().numpy().astype(np.float64)
        return np.linalg.norm(U.T @ U - np.eye(U.shape[1]))

    assert orth(U32) < 5e-5 and orth(U16) > 10 * orth(U32), (orth(U32), orth(U16))

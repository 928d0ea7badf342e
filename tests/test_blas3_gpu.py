"""rsyrk / rtrsm / rtrmm / rpotrf on the GPU against the oracle and FP64."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen, metrics
from oracle import later_oracle as lo

pytestmark = pytest.mark.gpu

# FP16 tensor-core updates: relative errors at the FP16 product level.
BOUND = {"fp16": 6e-4, "bf16": 6e-3, "split3": 3e-6}


def dev(x):
    return lg.colmajor(torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).cuda())


@pytest.mark.parametrize("n,k,prec", [(256, 128, "fp16"), (1000, 300, "fp16"), (2048, 2048, "fp16"),
                                      (777, 64, "bf16"), (1024, 512, "split3")])
def test_rsyrk(cuda, n, k, prec):
    A = gen.normal(n, k, seed=n + k)
    C0 = gen.normal(n, n, seed=7)
    dC = dev(C0)
    lg.later_rsyrk(n, k, -1.0, dev(A), 0.5, dC, precision=prec)
    assert lg.device_status() == 0
    C = dC.cpu().numpy()
    ref = lo.rsyrk(-1.0, A, 0.5, C0, prec)
    il = np.tril_indices(n)
    err = np.linalg.norm(C[il] - ref[il]) / np.linalg.norm(ref[il])
    assert err < 1e-6 + 2e-7 * k ** 0.5, err
    iu = np.triu_indices(n, 1)
    assert np.array_equal(C[iu], C0[iu])  # strictly upper triangle untouched


def _spd_chol(n, seed):
    return np.linalg.cholesky(gen.spd_matrix(n, 1e2, seed).astype(np.float64)).astype(np.float32)


@pytest.mark.parametrize("m,n", [(300, 128), (2048, 1024), (1000, 600), (4096, 256)])
def test_rtrsm_right_lower_trans(cuda, m, n):
    L = _spd_chol(n, 1)
    B = gen.normal(m, n, seed=2)
    dB = dev(B)
    lg.later_rtrsm("l", "r", "t", m, n, dev(L), dB)
    assert lg.device_status() == 0
    X = dB.cpu().numpy().astype(np.float64)
    bwd = np.linalg.norm(X @ L.T.astype(np.float64) - B) / np.linalg.norm(B)
    Xo = lo.rtrsm("r", L, B)
    bwd_o = np.linalg.norm(Xo.astype(np.float64) @ L.T.astype(np.float64) - B) / np.linalg.norm(B)
    assert bwd < max(3 * bwd_o, 1e-6) and bwd < BOUND["fp16"], (bwd, bwd_o)


@pytest.mark.parametrize("m,n", [(128, 300), (1024, 2048), (600, 1000)])
def test_rtrsm_left_lower_notrans(cuda, m, n):
    L = _spd_chol(m, 3)
    B = gen.normal(m, n, seed=4)
    dB = dev(B)
    lg.later_rtrsm("l", "l", "n", m, n, dev(L), dB)
    assert lg.device_status() == 0
    X = dB.cpu().numpy().astype(np.float64)
    bwd = np.linalg.norm(L.astype(np.float64) @ X - B) / np.linalg.norm(B)
    assert bwd < BOUND["fp16"], bwd


def test_rtrsm_reference_constant_input(cuda):
    # test/test_trsm.cu:44-66: L = lower triangle of 0.1, B = ones * L, solve X L^T = B.
    m, n = 2048, 1024
    L = gen.lower_tri_const(n)
    B = (np.ones((m, n), np.float32) @ L).astype(np.float32)
    dB = dev(B)
    lg.later_rtrsm("l", "r", "t", m, n, dev(L), dB)
    assert lg.device_status() == 0
    X = dB.cpu().numpy().astype(np.float64)
    bwd = np.linalg.norm(X @ L.T.astype(np.float64) - B) / np.linalg.norm(B)
    Xo = lo.rtrsm("r", L, B)
    bwd_o = np.linalg.norm(Xo.astype(np.float64) @ L.T.astype(np.float64) - B) / np.linalg.norm(B)
    assert bwd < max(3 * bwd_o, 1e-6), (bwd, bwd_o)


def test_rtrsm_unsupported_flags(cuda):
    L, B = dev(np.eye(64)), dev(np.ones((64, 64)))
    with pytest.raises(lg.LaterError) as e:
        lg.later_rtrsm("u", "l", "n", 64, 64, L, B)
    assert e.value.status == 5


@pytest.mark.parametrize("m,n", [(128, 100), (1000, 300), (2048, 2048)])
def test_rtrmm(cuda, m, n):
    L = _spd_chol(m, 5)
    B = gen.normal(m, n, seed=6)
    dC = dev(np.zeros((m, n)))
    lg.later_rtrmm(m, n, dev(L), dev(B), dC)
    assert lg.device_status() == 0
    ref = np.tril(L).astype(np.float64) @ B
    err = np.linalg.norm(dC.cpu().numpy() - ref) / np.linalg.norm(ref)
    err_o = np.linalg.norm(lo.rtrmm(L, B) - ref) / np.linalg.norm(ref)  # the reference's arithmetic
    assert err < max(3 * err_o, 1e-6) and err < BOUND["fp16"], (err, err_o)


@pytest.mark.parametrize("n,kappa,prec", [(100, 1e2, "fp16"), (250, 1e3, "fp16"), (256, 1e2, "fp16"),
                                          (1024, 1e2, "fp16"), (4096, 1e2, "fp16"),
                                          (2000, 1e2, "bf16"), (2048, 1e6, "split3"), (6144, 1e2, "fp16"),
                                          (4096, 1e4, "bf16")])
def test_rpotrf(cuda, n, kappa, prec):
    A = gen.spd_matrix(n, kappa, seed=n)
    dA = dev(A)
    lg.later_rpotrf("l", n, dA, precision=prec)
    assert lg.device_status() == 0
    L = np.tril(dA.cpu().numpy())
    bwd = metrics.chol_backward_error(A, L)
    # the oracle's restatement of l_potrf (FP32 leaves up to 2048, FP16 trsm / syrk updates above)
    bwd_o = metrics.chol_backward_error(A, lo.rpotrf(A, prec=prec))
    assert bwd < max(3 * bwd_o, 1e-6) and bwd < BOUND[prec], (bwd, bwd_o)
    # strictly upper triangle untouched
    iu = np.triu_indices(n, 1)
    assert np.array_equal(dA.cpu().numpy()[iu], A[iu])


def test_rpotrf_reference_constant_input(cuda):
    # test/test_potrf.cu:38-62: A = T T^T with T the lower triangle of 0.1.
    n = 1024
    T = gen.lower_tri_const(n).astype(np.float64)
    A = (T @ T.T).astype(np.float32)
    dA = dev(A)
    lg.later_rpotrf("l", n, dA)
    assert lg.device_status() == 0
    L = np.tril(dA.cpu().numpy())
    assert metrics.chol_backward_error(A, L) < BOUND["fp16"]


def test_rpotrf_not_spd_reports_numeric(cuda):
    n = 512
    A = -np.eye(n, dtype=np.float32)
    dA = dev(A)
    lg.later_rpotrf("l", n, dA)
    assert lg.device_status() == 7  # LATER_ERR_NUMERIC
    assert lg.device_status() == 0  # cleared

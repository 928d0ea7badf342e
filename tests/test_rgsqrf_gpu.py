"""later_rgsqrf on the GPU against the oracle restatement and FP64 LAPACK, same seeded inputs."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen, metrics
from oracle import later_oracle as lo

pytestmark = pytest.mark.gpu

# Accuracy bounds per precision (FP64-measured). The GPU result must be within
# a factor FACTOR of the oracle's own figure and below the absolute bound.
FACTOR = 3.0
BOUND_BWD = {"fp16": 5e-4, "bf16": 4e-3, "split3": 2e-6}


def run_gpu(A, **kw):
    dA = lg.colmajor(torch.from_numpy(np.ascontiguousarray(A)).cuda())
    R = lg.later_rgsqrf(dA, **kw)
    assert lg.device_status() == 0
    return dA.cpu().numpy(), R.cpu().numpy()


@pytest.mark.parametrize("m,n,leaf,prec,cgs2", [
    (1024, 128, 128, "fp16", False),
    (1024, 256, 128, "fp16", False),
    (4096, 1024, 128, "fp16", False),
    (2048, 512, 64, "fp16", False),
    (1000, 256, 32, "fp16", False),
    (3001, 384, 128, "bf16", False),
    (2048, 512, 128, "split3", False),
    (2048, 512, 128, "fp16", True),
    (300, 96, 128, "fp16", False),
    (70000, 64, 64, "fp16", False),
])
def test_rgsqrf_matches_oracle(cuda, m, n, leaf, prec, cgs2):
    A = gen.normal(m, n, seed=m + n)
    Q, R = run_gpu(A, leaf=leaf, precision=prec, cgs2=cgs2)
    Qo, Ro = lo.rgsqrf(A, leaf=leaf, prec=prec, cgs2=cgs2)
    bwd, orth = metrics.qr_backward_error(A, Q, R), metrics.orthogonality(Q)
    bwd_o, orth_o = metrics.qr_backward_error(A, Qo, Ro), metrics.orthogonality(Qo)
    assert bwd <= max(FACTOR * bwd_o, 1e-6) and bwd <= BOUND_BWD[prec], (bwd, bwd_o)
    assert orth <= max(FACTOR * orth_o, 1e-5), (orth, orth_o)
    # R upper triangular with positive diagonal and zeros below; close to the oracle's R.
    assert np.all(np.tril(R, -1) == 0)
    assert np.all(np.diag(R) > 0)
    assert np.linalg.norm(R - Ro) / np.linalg.norm(Ro) <= max(FACTOR * BOUND_BWD[prec], 1e-5)


def test_rgsqrf_uniform_reference_input(cuda):
    # The reference's test input distribution: U(0,1) (util/util.cu:102-109).
    A = gen.uniform(2048, 256, seed=3000)
    Q, R = run_gpu(A)
    Qx, Rx = metrics.lapack_qr_positive(A)
    assert metrics.qr_backward_error(A, Q, R) < 2e-4
    assert np.linalg.norm(R - Rx) / np.linalg.norm(Rx) < 2e-4


def test_rgsqrf_deterministic(cuda):
    A = gen.normal(4096, 512, seed=9)
    Q1, R1 = run_gpu(A)
    Q2, R2 = run_gpu(A)
    assert np.array_equal(Q1, Q2) and np.array_equal(R1, R2)


def test_rgsqrf_lda_larger_than_m(cuda):
    m, n = 1500, 256
    A = gen.normal(m, n, seed=4)
    dA = lg.empty_colmajor(m, n, ld=m + 36)
    dA.copy_(torch.from_numpy(A).cuda())
    R = lg.later_rgsqrf(dA)
    assert lg.device_status() == 0
    Q = dA.cpu().numpy()
    assert metrics.qr_backward_error(A, Q, R.cpu().numpy()) < 5e-4


def test_rgsqrf_rejects_bad_args(cuda):
    A = lg.empty_colmajor(100, 200)
    with pytest.raises(lg.LaterError):
        lg.later_rgsqrf(A)  # m < n


@pytest.mark.parametrize("m,n", [(1000, 100), (700, 17), (4096, 333)])
def test_rgsqrf_any_width(cuda, m, n):
    A = gen.normal(m, n, seed=n)
    Q, R = run_gpu(A)
    Qo, Ro = lo.rgsqrf(A)
    assert metrics.qr_backward_error(A, Q, R) <= max(3 * metrics.qr_backward_error(A, Qo, Ro), 1e-6)
    assert metrics.orthogonality(Q) <= max(3 * metrics.orthogonality(Qo), 1e-5)
    assert np.all(np.tril(R, -1) == 0) and np.all(np.diag(R) > 0)

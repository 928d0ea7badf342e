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
BOUND_BWD = {"fp16": 5e-4, "bf16": 4e-3, "split3": 2e-6, "split2": 2e-6}


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
    (4096, 1024, 128, "split2", False),
    (1000, 256, 32, "split2", False),
    (2048, 512, 128, "split2", True),
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
    # split2 keeps R12 at its FP16 value: R agrees with the oracle's to FP16 level, like fp16.
    r_tol = FACTOR * BOUND_BWD["fp16"] if prec == "split2" else max(FACTOR * BOUND_BWD[prec], 1e-5)
    assert np.linalg.norm(R - Ro) / np.linalg.norm(Ro) <= r_tol


def test_split2_backward_error_at_fp32_level(cuda):
    """split2 pays 1.5x the FP16 tensor work for an FP32-level backward error; FP16 stays near 1e-4."""
    A = gen.svd_matrix(4096, 1024, 1e3, seed=21)
    Q2, R2 = run_gpu(A, precision="split2")
    Qh, Rh = run_gpu(A, precision="fp16")
    b2, bh = metrics.qr_backward_error(A, Q2, R2), metrics.qr_backward_error(A, Qh, Rh)
    assert b2 <= 2e-6 and bh >= 20 * b2, (b2, bh)
    assert metrics.orthogonality(Q2) <= 2 * metrics.orthogonality(Qh) + 1e-5


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


@pytest.mark.parametrize("m,n", [(1000, 100), (700, 17), (4096, 333), (2000, 127)])
def test_rgsqrf_any_width(cuda, m, n):
    A = gen.normal(m, n, seed=n)
    Q, R = run_gpu(A)
    Qo, Ro = lo.rgsqrf(A)
    assert metrics.qr_backward_error(A, Q, R) <= max(3 * metrics.qr_backward_error(A, Qo, Ro), 1e-6)
    assert metrics.orthogonality(Q) <= max(3 * metrics.orthogonality(Qo), 1e-5)
    assert np.all(np.tril(R, -1) == 0) and np.all(np.diag(R) > 0)


@pytest.mark.parametrize("m,n,prec,cgs2", [(4096, 512, "fp16", False), (2048, 256, "split3", False),
                                           (16384, 128, "fp16", False), (3001, 200, "bf16", True)])
def test_fused_leaf_matches_mgs_panels(cuda, m, n, prec, cgs2):
    """The fused leaf (CholQR2 panels, one launch per leaf) and the reference's panel algorithm
    (MGS-TSQR, separate launches) give the same factorisation to working accuracy."""
    A = gen.normal(m, n, seed=7 + m)
    Qf, Rf = run_gpu(A, precision=prec, cgs2=cgs2)
    Qm, Rm = run_gpu(A, precision=prec, cgs2=cgs2, panel="mgs")
    for Q, R in ((Qf, Rf), (Qm, Rm)):
        assert metrics.qr_backward_error(A, Q, R) <= BOUND_BWD[prec]
        assert np.all(np.tril(R, -1) == 0) and np.all(np.diag(R) > 0)
    assert np.linalg.norm(Rf - Rm) / np.linalg.norm(Rm) <= 2 * BOUND_BWD[prec]
    assert metrics.orthogonality(Qf) <= 2 * metrics.orthogonality(Qm) + 1e-5


@pytest.mark.parametrize("kappa,prec", [(1e3, "fp16"), (1e5, "fp16"), (1e5, "split3"), (1e5, "split2")])
def test_fused_leaf_ill_conditioned(cuda, kappa, prec):
    """SVD-constructed inputs (the precision sweep's construction): the fused leaf, whose right-looking
    panels take their first-pass Gram matrix from the previous panel's reduction, keeps the backward
    error and orthogonality of the reference's MGS-TSQR panels."""
    A = gen.svd_matrix(4096, 512, kappa, seed=17)
    Qf, Rf = run_gpu(A, precision=prec)
    Qm, Rm = run_gpu(A, precision=prec, panel="mgs")
    bf, bm = metrics.qr_backward_error(A, Qf, Rf), metrics.qr_backward_error(A, Qm, Rm)
    assert bf <= max(2 * bm, 1e-6) and bf <= BOUND_BWD[prec], (bf, bm)
    assert metrics.orthogonality(Qf) <= 2 * metrics.orthogonality(Qm) + 1e-5
    assert np.all(np.tril(Rf, -1) == 0) and np.all(np.diag(Rf) > 0)


def test_fused_leaf_falls_back_on_dependent_columns(cuda):
    """Exactly dependent columns inside a 32-column panel break CholQR2 (a non-positive pivot, or a
    second Gram matrix far from I); that panel is factored by MGS-TSQR inside the same launch."""
    A = gen.normal(2048, 128, seed=11)
    A[:, 5] = A[:, 3]
    A[:, 70] = 2.0 * A[:, 69]
    Qf, Rf = run_gpu(A)
    Qm, Rm = run_gpu(A, panel="mgs")
    assert np.all(np.isfinite(Qf)) and np.all(np.isfinite(Rf))
    assert metrics.qr_backward_error(A, Qf, Rf) <= BOUND_BWD["fp16"]
    scale = np.linalg.norm(A, 2)
    assert abs(Rf[5, 5]) < 1e-2 * scale and abs(Rf[70, 70]) < 1e-2 * scale
    # MGS turns a dependent column into normalised rounding noise (so does the reference); the
    # orthogonality of the other columns is as good as with MGS-TSQR panels throughout.
    keep = [j for j in range(128) if j not in (5, 70)]

    def orth(Q):
        Qk = Q[:, keep].astype(np.float64)
        return np.linalg.norm(Qk.T @ Qk - np.eye(len(keep)))

    assert orth(Qf) <= 4 * orth(Qm) + 0.1, (orth(Qf), orth(Qm))
    # Panel 0 was factored by the fallback: the same MGS-TSQR arithmetic as the reference's path,
    # bit for bit (CholQR2 would round differently).
    assert np.array_equal(Qf[:, :32], Qm[:, :32]) and np.array_equal(Rf[:32, :32], Rm[:32, :32])


@pytest.mark.parametrize("m,n,prec", [(4096, 512, "fp16"), (2048, 256, "split3"), (16384, 128, "fp16"), (1000, 200, "bf16")])
def test_wide_leaf_matches_mgs_panels(cuda, m, n, prec):
    """panel = 2: one CholQR2 over each whole leaf when it is well conditioned (else 32-column
    panels): same factorisation as the reference's panel algorithm to working accuracy."""
    A = gen.normal(m, n, seed=5 + n)
    Qw, Rw = run_gpu(A, precision=prec, panel="wide")
    Qm, Rm = run_gpu(A, precision=prec, panel="mgs")
    assert metrics.qr_backward_error(A, Qw, Rw) <= BOUND_BWD[prec]
    assert np.all(np.tril(Rw, -1) == 0) and np.all(np.diag(Rw) > 0)
    assert np.linalg.norm(Rw - Rm) / np.linalg.norm(Rm) <= 2 * BOUND_BWD[prec]
    assert metrics.orthogonality(Qw) <= 2 * metrics.orthogonality(Qm) + 1e-5


def test_wide_leaf_falls_back_on_dependent_columns(cuda):
    """With exactly dependent columns the leaf-wide factorisation is refused and the leaf falls
    back to 32-column panels and, for the affected panel, to MGS-TSQR."""
    A = gen.normal(2048, 128, seed=11)
    A[:, 5] = A[:, 3]
    Qw, Rw = run_gpu(A, panel="wide")
    Qm, Rm = run_gpu(A, panel="mgs")
    assert np.all(np.isfinite(Qw)) and metrics.qr_backward_error(A, Qw, Rw) <= BOUND_BWD["fp16"]
    assert np.array_equal(Qw[:, :32], Qm[:, :32]) and np.array_equal(Rw[:32, :32], Rm[:32, :32])

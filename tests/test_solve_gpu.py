"""Mixed-precision SPD and least-squares solvers against FP64 LAPACK solutions."""
import numpy as np
import pytest
import torch

import later_gb300 as lg
from oracle import gen, metrics

pytestmark = pytest.mark.gpu


def dev(x, dtype=np.float32):
    return lg.colmajor(torch.from_numpy(np.ascontiguousarray(x, dtype=dtype)).cuda())


@pytest.mark.parametrize("n,kappa,prec,nrhs", [(1024, 1e2, "fp16", 16), (2048, 1e2, "fp16", 4),
                                               (2048, 1e6, "fp16", 16), (4096, 1e6, "fp16", 2),
                                               (1500, 1e6, "split3", 1), (777, 1e3, "bf16", 3)])
def test_spd_solve_refines_to_fp64_backward_error(cuda, n, kappa, prec, nrhs):
    A = gen.spd_matrix(n, kappa, seed=n)
    B = gen.normal(n, nrhs, seed=2)
    X, info = lg.spd_solve(dev(A), dev(B), precision=prec, max_iter=40, tol=1e-12)
    X = X.cpu().numpy()
    A64, B64 = A.astype(np.float64), B.astype(np.float64)
    # Normwise backward error (inf-norm form, as the solver's stopping test) in FP64 on the host.
    r = B64 - A64 @ X
    eta = max(np.abs(r[:, c]).max() / (np.abs(A64).sum(1).max() * np.abs(X[:, c]).max() + np.abs(B64[:, c]).max())
              for c in range(nrhs))
    assert eta <= 1e-12, (eta, info)
    assert info["backward_error"] <= 1e-12
    if kappa >= 1e6 and prec == "fp16" and n > 2048:
        # Above the 2048 FP32 block the trailing updates are FP16, whose Schur
        # complement at kappa 1e6 is not SPD: the solver refactors in SPLIT3.
        assert info["factor_precision"] == 2
    Xref = np.linalg.solve(A64, B64)
    assert np.linalg.norm(X - Xref) / np.linalg.norm(Xref) < kappa * 1e-11


@pytest.mark.parametrize("m,n,kappa,prec", [(4096, 512, 1e3, "split3"), (8192, 1024, 1e4, "split3"),
                                            (2048, 256, 1e1, "fp16"), (3000, 320, 1e2, "split3")])
def test_ls_solve_refines(cuda, m, n, kappa, prec):
    rng = np.random.default_rng(5)
    A = gen.svd_matrix(m, n, kappa, seed=m + n)
    xs = rng.standard_normal((n, 2))
    B = (A.astype(np.float64) @ xs + 1e-3 * rng.standard_normal((m, 2))).astype(np.float32)
    X, info = lg.ls_solve(dev(A), dev(B), precision=prec, max_iter=30, tol=1e-6)
    X = X.cpu().numpy()
    assert info["backward_error"] <= 1e-6, info
    A64 = A.astype(np.float64)
    Xref = np.linalg.lstsq(A64, B.astype(np.float64), rcond=None)[0]
    # Forward error within the LS perturbation bound for the reached backward error:
    # kappa + kappa^2 ||r|| / (||A|| ||x||) (Wedin). The solver's backward error is
    # the inf-norm augmented-system measure; converting it to the 2-norm relative
    # perturbation of A costs up to sqrt(m n), hence the factor 1000.
    rref = B.astype(np.float64) - A64 @ Xref
    s2 = np.linalg.norm(A64, 2)
    cond = kappa + kappa ** 2 * np.linalg.norm(rref) / (s2 * np.linalg.norm(Xref))
    fwd = np.linalg.norm(X - Xref) / np.linalg.norm(Xref)
    assert fwd < max(1000 * cond * info["backward_error"], 1e-6), (fwd, cond, info)
    # host FP64 check of the augmented-system backward error
    r = B.astype(np.float64) - A64 @ X
    g = A64.T @ r
    aug = max(1 + np.abs(A64).sum(1).max(), np.abs(A64).sum(0).max())
    eta = max(np.abs(g[:, c]).max() / (aug * max(np.abs(r[:, c]).max(), np.abs(X[:, c]).max()) + np.abs(B[:, c]).max())
              for c in range(2))
    assert eta <= 2e-6, eta


def test_ls_refinement_reduces_the_backward_error(cuda):
    # Well-conditioned LS with a tight tolerance: refinement must take steps and
    # push the FP64 backward error below what the factorisation alone gives.
    m, n = 4096, 256
    rng = np.random.default_rng(9)
    A = gen.svd_matrix(m, n, 10.0, seed=1)
    B = (A.astype(np.float64) @ rng.standard_normal((n, 1)) + 1e-3 * rng.standard_normal((m, 1))).astype(np.float32)
    X0, i0 = lg.ls_solve(dev(A), dev(B), precision="fp16", max_iter=0, tol=0.0)
    X1, i1 = lg.ls_solve(dev(A), dev(B), precision="fp16", max_iter=20, tol=1e-9)
    assert i1["iterations"] >= 1
    assert i1["backward_error"] < i0["backward_error"] / 10, (i0, i1)

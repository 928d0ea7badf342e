"""The precision sweep's error estimator (bench.py: qr_errors_probe), checked on the CPU.

The sweep reports ||A - QR||_F / ||A||_F and ||I - Q^T Q||_F estimated in FP64 from k Gaussian probe
vectors X: E ||E X||_F^2 = k ||E||_F^2, so the estimate's relative spread is about sqrt(2 / k). Here a
QR perturbed by known amounts is measured both ways; with k = 64 the estimates must land within 40% of
the exact FP64 norms (about 2.2 standard deviations), on several seeds.
"""
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_probe_estimates_match_exact_norms(seed):
    rng = np.random.default_rng(seed)
    m, n, k = 600, 80, 64
    A = rng.standard_normal((m, n))
    Q, R = np.linalg.qr(A)
    # perturb both factors: a backward error near 1e-5 and a loss of orthogonality near 1e-6
    Qp = Q + 1e-6 * rng.standard_normal((m, n)) / np.sqrt(m)
    Rp = R + 1e-5 * np.linalg.norm(A) / n * np.triu(rng.standard_normal((n, n)))
    exact_bwd = np.linalg.norm(A - Qp @ np.triu(Rp)) / np.linalg.norm(A)
    exact_orth = np.linalg.norm(np.eye(n) - Qp.T @ Qp)
    A0d = torch.from_numpy(A)
    X = torch.from_numpy(rng.standard_normal((n, k)))
    bwd, orth = bench.qr_errors_probe(A0d, A0d @ X, X, torch.from_numpy(Qp).float(), torch.from_numpy(Rp).float())
    # the FP32 rounding of Q and R (about 6e-8 relative) is far below the planted errors
    assert abs(bwd / exact_bwd - 1.0) < 0.4, (bwd, exact_bwd)
    assert abs(orth / exact_orth - 1.0) < 0.4, (orth, exact_orth)

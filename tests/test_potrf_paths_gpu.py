"""rpotrf's alternative schedules give the same factor to the arithmetic's accuracy.

A block of at most 2048 columns (the size the reference hands to cuSOLVER's FP32
Spotrf, Cholesky/later_rpotrf.cu:26-35) is by default factored by the blocked
right-looking loop: per 128-column block the Cholesky leaf, one solve launch for
every row below and one SPLIT3 lower-triangle update. A process started with
LATER_POTRF_BLOCKED=0 factors it by the split-in-half recursion instead. Both are
FP32-level: on the same input the blocked factor's FP64 backward error is at most
twice the recursion's (it is usually smaller: fewer roundings of each update), both
are within the FP32-level bound of the SPLIT3 tests, and the two factors agree far
below FP16 rounding. The 256-column inverse solves above 2048 columns have their own
switch and test below.
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import gen, metrics
from oracle import later_oracle as lo

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
BOUND_FP32_LEVEL = 3e-6  # the SPLIT3 bound of the BLAS-3 and Cholesky tests

SCRIPT = r"""
import sys
import numpy as np
import torch
import later_gb300 as lg

def run(A, prec):
    n = A.shape[0]
    dA = lg.colmajor(torch.from_numpy(np.ascontiguousarray(A)).cuda())
    lg.later_rpotrf("l", n, dA, precision=prec)
    assert lg.device_status() == 0
    return np.tril(dA.cpu().numpy())

if __name__ == "__main__":
    d = np.load(sys.argv[1])
    np.save(sys.argv[2], run(d["A"], str(d["prec"])))
"""


def _factor_both_ways(tmp_path, A, prec, switch):
    """The factor in this process (defaults) and in a child process with `switch`=0."""
    script = tmp_path / "potrf_case.py"
    script.write_text(SCRIPT)
    np.savez(tmp_path / "in.npz", A=A, prec=prec)
    env = dict(os.environ, PYTHONPATH=str(ROOT) + os.pathsep + os.environ.get("PYTHONPATH", ""))
    env[switch] = "0"
    out = tmp_path / "off.npy"
    r = subprocess.run([sys.executable, str(script), str(tmp_path / "in.npz"), str(out)], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    sys.path.insert(0, str(tmp_path))
    try:
        import potrf_case
        L_on = potrf_case.run(A, prec)
    finally:
        sys.path.remove(str(tmp_path))
        sys.modules.pop("potrf_case", None)
    return L_on, np.load(out)


def _rel(L, L0):
    return np.linalg.norm(L.astype(np.float64) - L0) / np.linalg.norm(L0.astype(np.float64))


@pytest.mark.parametrize("n,kappa,prec", [(2048, 1e2, "fp16"), (1000, 1e4, "fp16"), (3000, 1e2, "split3")])
def test_blocked_and_recursive_schedules_agree(cuda, tmp_path, n, kappa, prec):
    A = gen.spd_matrix(n, kappa, seed=n + 5)
    L_blk, L_rec = _factor_both_ways(tmp_path, A, prec, "LATER_POTRF_BLOCKED")
    b_blk = metrics.chol_backward_error(A, L_blk)
    b_rec = metrics.chol_backward_error(A, L_rec)
    b_or = metrics.chol_backward_error(A, lo.rpotrf(A, prec=prec))
    assert b_blk <= 2.0 * b_rec + 1e-8, (b_blk, b_rec)
    assert max(b_blk, b_rec) <= max(3.0 * b_or, BOUND_FP32_LEVEL), (b_blk, b_rec, b_or)
    # below 2048 columns both are FP32-level: the factors agree far below FP16 rounding
    assert _rel(L_blk, L_rec) <= 1e-4 * np.sqrt(kappa)


@pytest.mark.parametrize("n,kappa,prec", [(4096, 1e2, "fp16"), (8192, 1e3, "bf16")])
def test_solves_against_256_column_inverses(cuda, tmp_path, n, kappa, prec):
    """Above 2048 columns the off-diagonal solves with at least 2048 rows are products with inverses of
    the factor's diagonal blocks. A 256-column solve whose two 128-column halves are inverted is one
    product with the 256 x 256 inverse (built from the halves' inverses); LATER_POTRF_INV256=0 keeps the
    two half-block products and the update between them. Same arithmetic level: backward errors within
    a factor of two, at or below the oracle's level, the factors equal to within the top levels'
    16-bit rounding."""
    A = gen.spd_matrix(n, kappa, seed=n + 9)
    L_on, L_off = _factor_both_ways(tmp_path, A, prec, "LATER_POTRF_INV256")
    b_on = metrics.chol_backward_error(A, L_on)
    b_off = metrics.chol_backward_error(A, L_off)
    b_or = metrics.chol_backward_error(A, lo.rpotrf(A, prec=prec))
    assert b_on <= 2.0 * b_off + 1e-8 and b_off <= 2.0 * b_on + 1e-8, (b_on, b_off)
    assert b_on <= 3.0 * b_or, (b_on, b_or)
    assert _rel(L_on, L_off) <= (2e-3 if prec == "fp16" else 1.6e-2), _rel(L_on, L_off)

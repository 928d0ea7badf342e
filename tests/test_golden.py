"""The oracle against golden vectors produced by the reference LATER itself (CPU; no GPU needed).

tests/golden/*.npz were generated by tests/golden/make_golden.py: the reference's own kernels (compiled
from its sources) and its host recursion with cuBLAS / cuSOLVER, run on a GB300, on inputs rebuilt here
from the recorded generator and seed. The oracle's restatement must reproduce them:
- the 128-column leaf (FP32 MGS-TSQR panels and FP32 block-CGS glue) entry by entry to FP32 rounding;
- the FP16 recursion to the size of one FP16 rounding of an operand, with the same FP64 errors;
- the Cholesky (FP32 leaves, FP16 trsm / syrk updates) on sampled entries and column norms.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import gen, metrics
from oracle import later_oracle as lo

GOLDEN = Path(__file__).resolve().parent / "golden"


def _load(name):
    p = GOLDEN / f"{name}.npz"
    if not p.exists():
        pytest.skip(f"missing golden fixture {p.name} (tests/golden/make_golden.py writes it on a GPU)")
    return np.load(p)


@pytest.mark.parametrize("name", ["rgsqrf_leaf_512x128", "rgsqrf_leaf_2600x128"])
def test_oracle_leaf_matches_reference_output(name):
    f = _load(name)
    A = gen.normal(int(f["m"]), int(f["n"]), int(f["seed"]))
    Qo, Ro = lo.rgsqrf(A)
    assert np.abs(Qo - f["Q"]).max() <= 2e-5 * np.abs(f["Q"]).max()
    assert np.abs(np.triu(Ro) - f["R"]).max() <= 2e-5 * np.abs(f["R"]).max()
    assert metrics.qr_backward_error(A, Qo, Ro) <= 3 * float(f["backward_error"]) + 1e-7


def test_oracle_fp16_recursion_matches_reference_output():
    f = _load("rgsqrf_fp16_512x256")
    A = gen.normal(int(f["m"]), int(f["n"]), int(f["seed"]))
    Qo, Ro = lo.rgsqrf(A, prec="fp16")
    assert np.linalg.norm(Qo - f["Q"]) / np.linalg.norm(f["Q"]) <= 2e-3
    assert np.linalg.norm(np.triu(Ro) - f["R"]) / np.linalg.norm(f["R"]) <= 2e-3
    b, b_ref = metrics.qr_backward_error(A, Qo, Ro), float(f["backward_error"])
    o, o_ref = metrics.orthogonality(Qo), float(f["orthogonality"])
    assert 0.5 * b_ref <= b <= 2 * b_ref, (b, b_ref)
    assert 0.5 * o_ref <= o <= 2 * o_ref + 1e-6, (o, o_ref)


def test_oracle_rpotrf_matches_reference_output():
    f = _load("rpotrf_fp16_4096")
    assert int(f["info"]) == 0
    A = gen.spd_matrix(int(f["n"]), float(f["kappa"]), int(f["seed"]))
    L = lo.rpotrf(A, prec="fp16")
    assert np.abs(L[::64, ::64] - f["L_sample"]).max() <= 2e-3 * np.abs(f["L_sample"]).max()
    norms = np.linalg.norm(L.astype(np.float64), axis=0)
    assert np.abs(norms - f["L_col_norms"]).max() <= 1e-3 * f["L_col_norms"].max()
    b, b_ref = metrics.chol_backward_error(A, L), float(f["backward_error"])
    assert 0.33 * b_ref <= b <= 3 * b_ref, (b, b_ref)

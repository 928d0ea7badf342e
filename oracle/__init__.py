"""CPU oracle for the recursive QR / Cholesky hot path — test infrastructure only.

`oracle.later_oracle` restates the reference's algorithms (LATER: QR/later_rgsqrf.cu,
QR/panel.cu, ...) in numpy, with the same precision behaviour (FP32 storage,
FP16-rounded tensor-core GEMM operands, FP32 accumulation); `oracle.metrics`
computes FP64 accuracy figures; `oracle.gen` makes the seeded inputs.

Only tests, `__graft_entry__.smoke()` and `bench.py`'s CPU baseline use this
package, and only as the checker: the product path never imports it.

Parity pinning: the reference ships no golden vectors and its tests assert
nothing. Its code is CUDA + cuBLAS/cuSOLVER, so it runs only on a GPU:
`oracle/build_ref.py` compiles its own device kernels from its sources into
cubins and `oracle/ref_harness.cu` drives them with its host recursion
restated call for call (`oracle/_ref`). The restatement here is pinned to that
reference run by (a) golden vectors it produced on a GB300
(tests/golden/*.npz, checked on the CPU by tests/test_golden.py) and (b) GPU
tests that compare the two on the same seeded inputs
(tests/test_ref_parity_gpu.py); and, independently of the reference, by the
uniqueness of the QR factorisation with a positive diagonal (LAPACK dgeqrf in
FP64) and closed-form answers on the reference tests' constant inputs
(test/test_trsm.cu:44-56, test/test_trmm.cu:43-55, test/test_potrf.cu:38-62).
"""

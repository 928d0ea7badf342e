"""CPU oracle for the recursive QR / Cholesky hot path — test infrastructure only.

`oracle.later_oracle` restates the reference's algorithms (LATER: QR/later_rgsqrf.cu,
QR/panel.cu, ...) in numpy, with the same precision behaviour (FP32 storage,
FP16-rounded tensor-core GEMM operands, FP32 accumulation); `oracle.metrics`
computes FP64 accuracy figures; `oracle.gen` makes the seeded inputs.

Only tests, `__graft_entry__.smoke()` and `bench.py`'s CPU baseline use this
package, and only as the checker: the product path never imports it.

Parity pinning: the reference ships no golden vectors or known-answer files,
and its code is CUDA + cuBLAS/cuSOLVER that needs a GPU and its own sources to
run, so its outputs cannot be produced here. The restatement is pinned instead
by (a) the uniqueness of the QR factorisation with a positive diagonal, checked
against LAPACK dgeqrf in FP64, (b) closed-form answers for the reference tests'
constant inputs (test/test_trsm.cu:44-56, test/test_trmm.cu:43-55,
test/test_potrf.cu:38-62), and (c) committed fixtures in tests/golden/.
Parity against the reference's own binaries is therefore "unpinned".
"""

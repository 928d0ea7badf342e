// Fused rgsqrf leaf (leaf.cu): the whole m x w leaf (w <= 128) in one
// cooperative launch.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "panel.cuh"
#include "runtime.cuh"

namespace later {

constexpr int kLeafMaxWidth = 128;
constexpr int kLeafSyncInts = 4;  // arrive, exit, abort, spare: zero before the first launch, zero after each

// Workspace (floats) of leaf_fused for an m-row leaf, including the MGS-TSQR
// fallback's tree stacks.
int64_t leaf_fused_work(int m);

// Q R of the m x w leaf A (w <= 128): Q overwrites A (FP32) and its 16-bit
// copy (qh / ql at ldh, may be null); R (w x w, upper, zeros below) goes to R.
// Each 32-column panel is factored by CholQR2 (Gram, Cholesky, triangular
// solve, twice); a panel whose Cholesky breaks down or whose second Gram
// matrix is far from the identity is factored by MGS-TSQR instead, inside the
// same launch. Panels are right-looking: each projects all later columns of
// the leaf in its second reduction (block MGS order). With cgs2 they are glued
// by block Gram-Schmidt updates in the order of the recursive split, each
// applied twice. `sync` points to
// kLeafSyncInts zeroed ints; `tsqr_counters` to zeroed TSQR tree counters.
// Returns LATER_ERR_NOT_SUPPORTED when the device cannot run the cooperative
// launch (the caller then uses the multi-launch leaf).
later_status_t leaf_fused(cudaStream_t st, int m, int w, float* A, int64_t lda, float* R, int64_t ldr, void* qh,
                          void* ql, int64_t ldh, int out_prec, int cgs2, bool try_wide, Arena& ws, int* sync,
                          int* tsqr_counters, long long budget, int* fallbacks);

}  // namespace later

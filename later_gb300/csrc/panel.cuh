// Interfaces of the FP32 panel kernels (panel.cu) used by the drivers.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "runtime.cuh"

namespace later {

constexpr int kMaxTsqrLevels = 8;

// One TSQR tree over an m x 32 panel. Level 0 is the panel itself; level
// L >= 1 is the stack of the 32x32 R factors of level L-1 (32 rows per block).
struct TsqrPlan {
  int nlev;
  int maxbr;                      // tallest block of any level
  int br[kMaxTsqrLevels];         // rows per block at level L (256, 512 or 1024)
  int div[kMaxTsqrLevels];        // level-0 blocks per level-L block
  float* lev[kMaxTsqrLevels];
  int64_t ld[kMaxTsqrLevels];
  int rows[kMaxTsqrLevels];
  int nblk[kMaxTsqrLevels];
  int cnt_off[kMaxTsqrLevels];
  int* counters;
  float* R;
  int64_t ldr;
  int* status;
  long long budget;
  int ncols;  // columns of the level-0 panel (<= 32)
};

void tsqr_plan_sizes(int m, TsqrPlan* P, int64_t* stack_floats, int* ncounters);

// QR of the m x ncols panel A (ncols <= 32): Q overwrites A (FP32) and is also
// written to the 16-bit copy (qh / ql, may be null); R (ncols x ncols, upper)
// goes to R.
later_status_t tsqr_panel(cudaStream_t s, int m, float* A, int64_t lda, float* R, int64_t ldr, void* qh, void* ql,
                          int64_t ldh, int out_prec, Arena& ws, int* counters_zeroed, long long budget,
                          int ncols = 32);

// R = alpha X^T Y (+ R when accumulate) for X (m x k1), Y (m x k2), FP32
// (SIMT, deterministic split over rows).
later_status_t simt_tn(cudaStream_t s, int m, int k1, int k2, const float* X, int64_t ldx, const float* Y,
                       int64_t ldy, float* R, int64_t ldr, int accumulate, Arena& ws, float alpha = 1.f);

// Y -= X S for X (m x k1), S (k1 x k2), FP32 (SIMT); optional 16-bit copy of
// the updated Y (yh / yl with leading dimension ldh, format out_prec).
later_status_t simt_nn_sub(cudaStream_t s, int m, int k1, int k2, const float* X, int64_t ldx, const float* S,
                           int64_t lds, float* Y, int64_t ldy, void* yh = nullptr, void* yl = nullptr,
                           int64_t ldh = 0, int out_prec = LATER_PREC_FP16);

// Y += alpha X op(S), op(S) = S (k1 x k2) or, with s_trans, the transpose of a
// stored k2 x k1 S; with `lower`, only Y[i][j], i >= j, is updated. FP32 SIMT.
later_status_t simt_gemm_acc(cudaStream_t s, int m, int k1, int k2, float alpha, const float* X, int64_t ldx,
                             const float* S, int64_t lds, int s_trans, int lower, float* Y, int64_t ldy,
                             void* yh = nullptr, void* yl = nullptr, int64_t ldh = 0, int out_prec = 0);

}  // namespace later

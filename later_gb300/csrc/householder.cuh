// Householder reconstruction (rhouqr leaf) and explicit-Q forming (ormqr).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "runtime.cuh"

namespace later {

// 32x32 U, 32x32 T and 32 signs of one leaf, in caller workspace.
struct HrScratch {
  float* U;
  float* T;
  float* s;
};

// A (m x nc, nc <= 32) holds the explicit Q of a TSQR panel and R its R.
// Overwrites A with Y (unit lower trapezoidal), writes W = Y T into W, flips
// the rows of R so that I - W Y^T has Q S as its first nc columns and
// (Q S)(S R) = Q R. Writes 16-bit copies of Y and W when yh / wh are given.
later_status_t householder_reconstruct(cudaStream_t st, int m, int nc, float* A, int64_t lda, float* W, int64_t ldw,
                                       float* R, int64_t ldr, void* yh, void* yl, void* wh, void* wl, int64_t ldh,
                                       int out_prec, HrScratch hr);

// Q = I - W Y1^T (first n columns of the compact-WY orthogonal factor), FP32.
later_status_t form_q(cudaStream_t st, int m, int n, const float* W, int64_t ldw, const float* Y, int64_t ldy,
                      float* Q, int64_t ldq);

}  // namespace later

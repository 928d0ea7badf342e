// Recursive BLAS-3 and Cholesky drivers (blas3.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "qr.cuh"
#include "runtime.cuh"

namespace later {

// Minimum 16-bit scratch (hwork, in 16-bit elements) of each routine.
int64_t rsyrk_hwork(int n, int k, const Options& o);
int64_t rtrsm_hwork(int m, int n, char leri, const Options& o);
int64_t rtrmm_hwork(int m, int n, const Options& o);
int64_t rpotrf_hwork(int n, const Options& o);
// FP32 scratch (work) that lets the GEMMs split K over idle SMs (optional).
int64_t splitk_work();

later_status_t rsyrk(cudaStream_t st, int n, int k, float alpha, const float* A, int64_t lda, float beta, float* C,
                     int64_t ldc, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o);
later_status_t rtrsm(cudaStream_t st, char uplo, char leri, char trans, int m, int n, const float* A, int64_t lda,
                     float* B, int64_t ldb, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o);
// rtrsm with the FP32 / tensor-core switch at `fp32_lim` (rtrsm uses the
// reference's 256; the solvers pass INT_MAX: all-FP32 updates).
later_status_t rtrsm_lim(cudaStream_t st, char uplo, char leri, char trans, int m, int n, const float* A,
                         int64_t lda, float* B, int64_t ldb, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                         const Options& o, int fp32_lim);
later_status_t rtrmm(cudaStream_t st, int m, int n, const float* A, int64_t lda, const float* B, int64_t ldb,
                     float* C, int64_t ldc, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                     const Options& o);
later_status_t rpotrf(cudaStream_t st, char uplo, int n, float* A, int64_t lda, float* work, int64_t lwork,
                      void* hwork, int64_t lhwork, const Options& o);

}  // namespace later

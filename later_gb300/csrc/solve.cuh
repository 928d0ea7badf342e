// Mixed-precision SPD and least-squares solvers (solve.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "qr.cuh"

namespace later {

struct SolveNeed {
  int64_t work = 0;   // floats
  int64_t hwork = 0;  // 16-bit elements
};

struct SolveInfo {
  int iterations = 0;         // refinement steps taken
  double backward_error = 0;  // final normwise backward error (FP64)
  int factor_precision = 0;   // precision the factorisation finally used
};

SolveNeed spd_solve_need(int n, int k, const Options& o);
SolveNeed ls_solve_need(int m, int n, int k, const Options& o);

later_status_t spd_solve(cudaStream_t st, int n, int k, const float* A, int64_t lda, const float* B, int64_t ldb,
                         double* X, int64_t ldx, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                         const Options& o, int max_iter, double tol, SolveInfo* info);

later_status_t ls_solve(cudaStream_t st, int m, int n, int k, const float* A, int64_t lda, const float* B,
                        int64_t ldb, double* X, int64_t ldx, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                        const Options& o, int max_iter, double tol, SolveInfo* info);

}  // namespace later

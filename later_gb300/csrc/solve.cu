// Mixed-precision solvers on top of the factorisations (no reference
// counterpart: LATER has factorisations only).
//
//   SPD  A X = B:   A = L L^T by rpotrf (FP16/BF16/SPLIT3 tensor-core
//                   updates), then FP64 iterative refinement:
//                     r = B - A X (FP64 on the GPU), d = L^-T L^-1 r (FP32),
//                     X += d (FP64), until the normwise backward error
//                     max_c ||r_c||_inf / (||A||_inf ||x_c||_inf + ||b_c||_inf) <= tol.
//                   If the FP16/BF16 factorisation meets a non-positive pivot
//                   (the FP16 Schur complement of an ill-conditioned SPD matrix
//                   need not be SPD) the matrix is refactored in SPLIT3.
//   LS   min ||A X - B||:  A = Q R by rgsqrf, X = R^-1 Q^T B (FP32), then
//                   X += R^-1 Q^T (B - A X) with the residual in FP64, until the
//                   backward error of the augmented system [I A; A^T 0][r; x] = [b; 0],
//                     max_c ||A^T r_c||_inf / (||A_aug||_inf max(||r_c||, ||x_c||)_inf + ||b_c||_inf),
//                   is <= tol (Carson, Higham and Pranesh, SIAM J. Sci. Comput. 2020).
// FP64 arithmetic runs only in the residual / A^T r kernels and the X update.
// Both solvers synchronise the stream between iterations (host convergence test).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "blas3.cuh"
#include "panel.cuh"
#include "qr.cuh"
#include "runtime.cuh"
#include "solve.cuh"

namespace later {

namespace {

constexpr int RR = 64;   // rows per CTA in the residual kernel
constexpr int RK = 16;   // right-hand sides per CTA
constexpr int XJ = 64;   // columns of A staged per step

// R = B - A X for A (m x n, FP32), X (n x k, FP64), B (m x k, FP32), R FP64.
__global__ void __launch_bounds__(256) resid64_kernel(int m, int n, int k, const float* __restrict__ A, int64_t lda,
                                                      const double* __restrict__ X, int64_t ldx,
                                                      const float* __restrict__ B, int64_t ldb, double* R,
                                                      int64_t ldr) {
  __shared__ double xs[XJ][RK + 1];
  const int r = blockIdx.x * RR + threadIdx.x % RR;
  const int cg = threadIdx.x / RR;  // 4 groups of 4 right-hand sides
  const int c0 = blockIdx.y * RK;
  double acc[4] = {0, 0, 0, 0};
  for (int j0 = 0; j0 < n; j0 += XJ) {
    __syncthreads();
    for (int e = threadIdx.x; e < XJ * RK; e += 256) {
      const int jj = e % XJ, c = e / XJ;
      xs[jj][c] = (j0 + jj < n && c0 + c < k) ? X[j0 + jj + static_cast<int64_t>(c0 + c) * ldx] : 0.0;
    }
    __syncthreads();
    if (r < m) {
      const int jn = min(XJ, n - j0);
#pragma unroll 4
      for (int jj = 0; jj < jn; ++jj) {
        const double a = static_cast<double>(A[r + static_cast<int64_t>(j0 + jj) * lda]);
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u] = fma(a, xs[jj][4 * cg + u], acc[u]);
      }
    }
  }
  if (r >= m) return;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int c = c0 + 4 * cg + u;
    if (c < k) R[r + static_cast<int64_t>(c) * ldr] = static_cast<double>(B[r + static_cast<int64_t>(c) * ldb]) - acc[u];
  }
}

// G = A^T R (n x k, FP64): one CTA per column of A, fixed-order block reduction.
__global__ void __launch_bounds__(256) atr64_kernel(int m, int k, const float* __restrict__ A, int64_t lda,
                                                    const double* __restrict__ R, int64_t ldr, double* G,
                                                    int64_t ldg) {
  __shared__ double red[8][RK];
  const int j = blockIdx.x;
  double acc[RK];
#pragma unroll
  for (int c = 0; c < RK; ++c) acc[c] = 0.0;
  for (int r = threadIdx.x; r < m; r += 256) {
    const double a = static_cast<double>(A[r + static_cast<int64_t>(j) * lda]);
#pragma unroll
    for (int c = 0; c < RK; ++c)
      if (c < k) acc[c] = fma(a, R[r + static_cast<int64_t>(c) * ldr], acc[c]);
  }
#pragma unroll
  for (int c = 0; c < RK; ++c)
    for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int c = 0; c < RK; ++c) red[w][c] = acc[c];
  __syncthreads();
  if (threadIdx.x < k) {
    double s = 0.0;
    for (int ww = 0; ww < 8; ++ww) s += red[ww][threadIdx.x];
    G[j + static_cast<int64_t>(threadIdx.x) * ldg] = s;
  }
}

// Row sums of |A| (for ||A||_inf) and column sums (for ||A||_1), FP64.
__global__ void abs_row_sums(int m, int n, const float* __restrict__ A, int64_t lda, double* out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  double s = 0.0;
  for (int j = 0; j < n; ++j) s += fabs(static_cast<double>(A[r + static_cast<int64_t>(j) * lda]));
  out[r] = s;
}
__global__ void abs_col_sums(int m, const float* __restrict__ A, int64_t lda, double* out) {
  __shared__ double red[8];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int r = threadIdx.x; r < m; r += 256) s += fabs(static_cast<double>(A[r + static_cast<int64_t>(j) * lda]));
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    out[j] = t;
  }
}

// Column-wise infinity norms of an m x k FP64 or FP32 block.
template <class T>
__global__ void col_inf_norms(int m, int k, const T* __restrict__ X, int64_t ldx, double* out) {
  __shared__ double red[8];
  const int c = blockIdx.x;
  double s = 0.0;
  for (int r = threadIdx.x; r < m; r += 256) s = fmax(s, fabs(static_cast<double>(X[r + static_cast<int64_t>(c) * ldx])));
  for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t = fmax(t, red[w]);
    out[c] = t;
  }
}

__global__ void max_reduce(int n, const double* __restrict__ x, double* out) {
  __shared__ double red[8];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) s = fmax(s, x[i]);
  for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t = fmax(t, red[w]);
    *out = t;
  }
}

__global__ void d2f(int m, int k, const double* __restrict__ X, int64_t ldx, float* Y, int64_t ldy) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  for (int c = blockIdx.y; c < k; c += gridDim.y) Y[r + static_cast<int64_t>(c) * ldy] = static_cast<float>(X[r + static_cast<int64_t>(c) * ldx]);
}
__global__ void f2d_acc(int m, int k, const float* __restrict__ X, int64_t ldx, double* Y, int64_t ldy, int acc) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  for (int c = blockIdx.y; c < k; c += gridDim.y) {
    const double v = static_cast<double>(X[r + static_cast<int64_t>(c) * ldx]);
    double* y = &Y[r + static_cast<int64_t>(c) * ldy];
    *y = acc ? *y + v : v;
  }
}
// Lower L = R^T from the upper triangle of R (n x n).
__global__ void upper_to_lower(int n, const float* __restrict__ R, int64_t ldr, float* L, int64_t ldl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int j = blockIdx.y; j < n; j += gridDim.y)
    L[i + static_cast<int64_t>(j) * ldl] = (i >= j) ? R[j + static_cast<int64_t>(i) * ldr] : 0.f;
}

dim3 g2(int m, int k) { return dim3((m + 255) / 256, std::min(k, 65535)); }

struct Norms {
  double* rows;   // m
  double* cols;   // n
  double* a_inf;  // 1
  double* a_one;  // 1
  double* xn;     // k
  double* bn;     // k
  double* rn;     // k
  double* gn;     // k
};

later_status_t launch_ok() { return cuda_status(cudaGetLastError()); }

// Host read of k doubles (synchronises).
later_status_t fetch(cudaStream_t st, const double* d, int k, std::vector<double>* out) {
  out->assign(k, 0.0);
  LATER_CHECK_CUDA(cudaMemcpyAsync(out->data(), d, sizeof(double) * k, cudaMemcpyDeviceToHost, st));
  LATER_CHECK_CUDA(cudaStreamSynchronize(st));
  return LATER_OK;
}

later_status_t device_status_sync(cudaStream_t st) {
  int* p = device_status_ptr();
  int v = 0;
  LATER_CHECK_CUDA(cudaMemcpyAsync(&v, p, sizeof(int), cudaMemcpyDeviceToHost, st));
  LATER_CHECK_CUDA(cudaStreamSynchronize(st));
  if (v) LATER_CHECK_CUDA(cudaMemsetAsync(p, 0, sizeof(int), st));
  if (v & DEV_TIMEOUT) return LATER_ERR_TIMEOUT;
  if (v & DEV_NUMERIC) return LATER_ERR_NUMERIC;
  if (v & DEV_RANGE) return LATER_ERR_RANGE;
  return LATER_OK;
}

// Scratch carved from `work` (FP32 words) for the solvers.
struct SolveWs {
  float* F;      // factor (n x n for SPD, m x n for LS)
  float* Lt;     // LS: R^T as a lower triangle (n x n)
  float* R;      // LS: R (n x n)
  float* v32;    // n x k
  float* r32;    // m x k (FP32 copy of the residual)
  double* r64;   // m x k
  double* g64;   // n x k
  Norms nm;
  float* rest;   // remaining work for the factorisation / solves
  int64_t rest_floats;
};

bool carve_solve(Arena& a, int m, int n, int k, bool ls, SolveWs* w) {
  w->F = a.take<float>(static_cast<size_t>(m) * n);
  w->Lt = ls ? a.take<float>(static_cast<size_t>(n) * n) : nullptr;
  w->R = ls ? a.take<float>(static_cast<size_t>(n) * n) : nullptr;
  w->v32 = a.take<float>(static_cast<size_t>(n) * k);
  w->r32 = a.take<float>(static_cast<size_t>(m) * k);
  w->r64 = a.take<double>(static_cast<size_t>(m) * k);
  w->g64 = a.take<double>(static_cast<size_t>(n) * k);
  w->nm.rows = a.take<double>(m);
  w->nm.cols = a.take<double>(n);
  w->nm.a_inf = a.take<double>(1);
  w->nm.a_one = a.take<double>(1);
  w->nm.xn = a.take<double>(k);
  w->nm.bn = a.take<double>(k);
  w->nm.rn = a.take<double>(k);
  w->nm.gn = a.take<double>(k);
  return !a.failed();
}

later_status_t matrix_norms(cudaStream_t st, int m, int n, const float* A, int64_t lda, Norms& nm, bool one) {
  abs_row_sums<<<(m + 255) / 256, 256, 0, st>>>(m, n, A, lda, nm.rows);
  note_launch();
  max_reduce<<<1, 256, 0, st>>>(m, nm.rows, nm.a_inf);
  note_launch();
  if (one) {
    abs_col_sums<<<n, 256, 0, st>>>(m, A, lda, nm.cols);
    note_launch();
    max_reduce<<<1, 256, 0, st>>>(n, nm.cols, nm.a_one);
    note_launch();
  }
  return launch_ok();
}

}  // namespace

// ------------------------------------------------------------------- sizes
SolveNeed spd_solve_need(int n, int k, const Options& o) {
  Arena a(nullptr, 0);
  SolveWs w;
  carve_solve(a, n, n, k, false, &w);
  SolveNeed s;
  Options o3 = o;
  o3.prec = LATER_PREC_SPLIT3;  // room for the SPLIT3 refactorisation
  s.work = static_cast<int64_t>(a.peak() / sizeof(float)) + 1024 + splitk_work();
  s.hwork = std::max(std::max(rpotrf_hwork(n, o3), rtrsm_hwork(n, k, 'l', o3)), rtrsm_hwork(n, k, 'l', o3));
  return s;
}

SolveNeed ls_solve_need(int m, int n, int k, const Options& o) {
  Arena a(nullptr, 0);
  SolveWs w;
  carve_solve(a, m, n, k, true, &w);
  const QrNeed q = rgsqrf_need(m, n, o);
  SolveNeed s;
  s.work = static_cast<int64_t>(a.peak() / sizeof(float)) + 1024 + std::max<int64_t>(q.rec_work, splitk_work() + 4096LL * 64);
  s.hwork = std::max(q.hwork, rtrsm_hwork(n, k, 'l', o));
  return s;
}

// ------------------------------------------------------------------- SPD
later_status_t spd_solve(cudaStream_t st, int n, int k, const float* A, int64_t lda, const float* B, int64_t ldb,
                         double* X, int64_t ldx, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                         const Options& o, int max_iter, double tol, SolveInfo* info) {
  if (n < 1 || k < 1 || k > RK || !A || !B || !X || lda < n || ldb < n || ldx < n) return LATER_ERR_INVALID_ARG;
  const SolveNeed need = spd_solve_need(n, k, o);
  if (!work || !hwork || lwork < need.work || lhwork < need.hwork) return LATER_ERR_WORKSPACE;
  Arena a(work, static_cast<size_t>(lwork) * sizeof(float));
  SolveWs w;
  if (!carve_solve(a, n, n, k, false, &w)) return LATER_ERR_WORKSPACE;
  const int64_t rest_n = static_cast<int64_t>(a.remaining() / sizeof(float)) - 128;
  if (rest_n < 4096) return LATER_ERR_WORKSPACE;
  float* rest = a.take<float>(rest_n);
  Options of = o;
  // Factor (refactor in SPLIT3 if the 16-bit factorisation is not SPD).
  later_status_t fs = LATER_OK;
  for (int attempt = 0; attempt < 2; ++attempt) {
    LATER_CHECK(copy2d(st, n, n, A, lda, w.F, n));
    LATER_CHECK(rpotrf(st, 'l', n, w.F, n, rest, rest_n, hwork, lhwork, of));
    fs = device_status_sync(st);
    if (fs != LATER_ERR_NUMERIC || of.prec == LATER_PREC_SPLIT3) break;
    of.prec = LATER_PREC_SPLIT3;
  }
  if (fs != LATER_OK) return fs;
  info->factor_precision = of.prec;
  // Triangular solves with few right-hand sides run in FP32 throughout: a
  // 16-bit operand would underflow for small residuals and overflow for the
  // large solutions of ill-conditioned systems, and tensor cores gain nothing
  // at nrhs <= 16.
  auto solve = [&](float* V) -> later_status_t {
    LATER_CHECK(rtrsm_lim(st, 'l', 'l', 'n', n, k, w.F, n, V, n, rest, rest_n, hwork, lhwork, of, 1 << 30));
    return rtrsm_lim(st, 'l', 'l', 't', n, k, w.F, n, V, n, rest, rest_n, hwork, lhwork, of, 1 << 30);
  };
  LATER_CHECK(matrix_norms(st, n, n, A, lda, w.nm, false));
  col_inf_norms<float><<<k, 256, 0, st>>>(n, k, B, ldb, w.nm.bn);
  note_launch();
  LATER_CHECK(copy2d(st, n, k, B, ldb, w.v32, n));
  LATER_CHECK(solve(w.v32));
  f2d_acc<<<g2(n, k), 256, 0, st>>>(n, k, w.v32, n, X, ldx, 0);
  note_launch();
  std::vector<double> an, xn, bn, rn;
  LATER_CHECK(fetch(st, w.nm.a_inf, 1, &an));
  LATER_CHECK(fetch(st, w.nm.bn, k, &bn));
  info->iterations = 0;
  for (int it = 0; it <= max_iter; ++it) {
    resid64_kernel<<<dim3((n + RR - 1) / RR, (k + RK - 1) / RK), 256, 0, st>>>(n, n, k, A, lda, X, ldx, B, ldb, w.r64, n);
    note_launch();
    col_inf_norms<double><<<k, 256, 0, st>>>(n, k, w.r64, n, w.nm.rn);
    note_launch();
    col_inf_norms<double><<<k, 256, 0, st>>>(n, k, X, ldx, w.nm.xn);
    note_launch();
    LATER_CHECK(fetch(st, w.nm.rn, k, &rn));
    LATER_CHECK(fetch(st, w.nm.xn, k, &xn));
    double eta = 0.0;
    for (int c = 0; c < k; ++c) eta = std::max(eta, rn[c] / (an[0] * xn[c] + bn[c]));
    info->backward_error = eta;
    if (eta <= tol || it == max_iter) break;
    d2f<<<g2(n, k), 256, 0, st>>>(n, k, w.r64, n, w.v32, n);
    note_launch();
    LATER_CHECK(solve(w.v32));
    f2d_acc<<<g2(n, k), 256, 0, st>>>(n, k, w.v32, n, X, ldx, 1);
    note_launch();
    info->iterations = it + 1;
  }
  return launch_ok();
}

// ------------------------------------------------------------------- LS
later_status_t ls_solve(cudaStream_t st, int m, int n, int k, const float* A, int64_t lda, const float* B,
                        int64_t ldb, double* X, int64_t ldx, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                        const Options& o, int max_iter, double tol, SolveInfo* info) {
  if (m < n || n < 1 || k < 1 || k > RK || !A || !B || !X || lda < m || ldb < m || ldx < n)
    return LATER_ERR_INVALID_ARG;
  const SolveNeed need = ls_solve_need(m, n, k, o);
  if (!work || !hwork || lwork < need.work || lhwork < need.hwork) return LATER_ERR_WORKSPACE;
  Arena a(work, static_cast<size_t>(lwork) * sizeof(float));
  SolveWs w;
  if (!carve_solve(a, m, n, k, true, &w)) return LATER_ERR_WORKSPACE;
  const int64_t rest_n = static_cast<int64_t>(a.remaining() / sizeof(float)) - 128;
  if (rest_n < 4096) return LATER_ERR_WORKSPACE;
  float* rest = a.take<float>(rest_n);
  Arena pa(rest, static_cast<size_t>(rest_n) * sizeof(float));
  // Q R = A (Q over the copy F), L = R^T for the solves with R.
  LATER_CHECK(copy2d(st, m, n, A, lda, w.F, m));
  LATER_CHECK(rgsqrf(st, m, n, w.F, m, w.R, n, rest, rest_n, hwork, lhwork, o));
  LATER_CHECK(device_status_sync(st));
  upper_to_lower<<<g2(n, n), 256, 0, st>>>(n, w.R, n, w.Lt, n);
  note_launch();
  info->factor_precision = o.prec;
  Options os = o;  // the solves with R run in FP32 (n <= 256) or the factorisation's precision
  if (os.prec == LATER_PREC_SPLIT2) os.prec = LATER_PREC_FP16;  // SPLIT2 is a QR-only mode
  auto apply = [&](const float* V /*m x k*/) -> later_status_t {
    // v32[:n] = Q^T V, then R x = v  <=>  L^T x = v with L = R^T
    LATER_CHECK(simt_tn(st, m, n, k, w.F, m, V, m, w.v32, n, 0, pa, 1.f));
    return rtrsm_lim(st, 'l', 'l', 't', n, k, w.Lt, n, w.v32, n, rest, rest_n, hwork, lhwork, os, 1 << 30);
  };
  LATER_CHECK(matrix_norms(st, m, n, A, lda, w.nm, true));
  col_inf_norms<float><<<k, 256, 0, st>>>(m, k, B, ldb, w.nm.bn);
  note_launch();
  LATER_CHECK(apply(B));
  f2d_acc<<<g2(n, k), 256, 0, st>>>(n, k, w.v32, n, X, ldx, 0);
  note_launch();
  std::vector<double> ainf, aone, xn, bn, rn, gn;
  LATER_CHECK(fetch(st, w.nm.a_inf, 1, &ainf));
  LATER_CHECK(fetch(st, w.nm.a_one, 1, &aone));
  LATER_CHECK(fetch(st, w.nm.bn, k, &bn));
  const double aug = std::max(1.0 + ainf[0], aone[0]);
  info->iterations = 0;
  for (int it = 0; it <= max_iter; ++it) {
    resid64_kernel<<<dim3((m + RR - 1) / RR, (k + RK - 1) / RK), 256, 0, st>>>(m, n, k, A, lda, X, ldx, B, ldb, w.r64, m);
    note_launch();
    atr64_kernel<<<n, 256, 0, st>>>(m, k, A, lda, w.r64, m, w.g64, n);
    note_launch();
    col_inf_norms<double><<<k, 256, 0, st>>>(m, k, w.r64, m, w.nm.rn);
    note_launch();
    col_inf_norms<double><<<k, 256, 0, st>>>(n, k, X, ldx, w.nm.xn);
    note_launch();
    col_inf_norms<double><<<k, 256, 0, st>>>(n, k, w.g64, n, w.nm.gn);
    note_launch();
    LATER_CHECK(fetch(st, w.nm.rn, k, &rn));
    LATER_CHECK(fetch(st, w.nm.xn, k, &xn));
    LATER_CHECK(fetch(st, w.nm.gn, k, &gn));
    double eta = 0.0;
    for (int c = 0; c < k; ++c) eta = std::max(eta, gn[c] / (aug * std::max(rn[c], xn[c]) + bn[c]));
    info->backward_error = eta;
    if (eta <= tol || it == max_iter) break;
    // d = R^-1 Q^T r
    d2f<<<g2(m, k), 256, 0, st>>>(m, k, w.r64, m, w.r32, m);
    note_launch();
    LATER_CHECK(apply(w.r32));
    f2d_acc<<<g2(n, k), 256, 0, st>>>(n, k, w.v32, n, X, ldx, 1);
    note_launch();
    info->iterations = it + 1;
  }
  return launch_ok();
}

}  // namespace later

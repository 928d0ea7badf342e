// QDWH polar decomposition A = U H (EVD/later_qdwh_polar.cu:24-110), the
// largest caller of rgsqrf in the reference: every iteration factors the
// (m + n) x n stack [sqrt(c) X; I] and forms one product Q1 Q2^T.
//
//   X0 = A / ||A||_F,  l0 <= sigma_min(X0)
//   repeat:  (a, b, c) from l (dynamically weighted Halley), l <- l (a + b l^2) / (1 + c l^2)
//            [sqrt(c) X; I] = [Q1; Q2] R                 (rgsqrf, CGS2)
//            X <- (b/c) X + (a - b/c)/sqrt(c) Q1 Q2^T     (tensor-core GEMM, X as the accumulator)
//   until 1 - l < tol1 and ||X_new - X||_F < tol1^(1/3)  (the reference's tol1 / tol3)
//   U = X;  H = (U^T A + A^T U) / 2
//
// Differences from the reference, all needed for a usable result:
//   * the stack's QR has condition number about sqrt(c) (1e4 and more in the
//     first steps), so Gram-Schmidt must reorthogonalise (CGS2) and project at
//     the FP32 level (SPLIT3) for Q to be orthonormal; with the reference's
//     plain FP16 rgsqrf the iterate stalls at FP16-level orthogonality;
//   * the stack is scaled by c^(-1/4) (Q is unchanged) so that both blocks
//     stay inside the FP16 range of the 16-bit operand copies;
//   * l0 is a guaranteed lower bound 1 / ||R0^{-1}||_F from a QR of X0 (or the
//     caller's), where the reference hard-codes 2.07e-4 / sqrt(n) (:38-39);
//   * symmetrising each iterate (generateNewU, :9-21) is an option for
//     symmetric A only (it is wrong for a general A), done out of place (the
//     reference's in-place kernel races across thread blocks);
//   * H is computed (the reference leaves it untouched).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "../../include/later_c.h"
#include "blas3.cuh"
#include "qr.cuh"
#include "runtime.cuh"

namespace later {
namespace {

constexpr int kNormBlocks = 512;

// Per-block partial sums of squares of (X - Y) (Y may be null), in FP64.
__global__ void sumsq_kernel(int m, int n, const float* __restrict__ X, int64_t ldx, const float* __restrict__ Y,
                             int64_t ldy, double* part) {
  __shared__ double ws[8];
  double s = 0.0;
  const int64_t total = static_cast<int64_t>(m) * n;
  for (int64_t e = blockIdx.x * 256LL + threadIdx.x; e < total; e += 256LL * gridDim.x) {
    const int64_t j = e / m, i = e - j * m;
    double v = X[i + j * ldx];
    if (Y) v -= Y[i + j * ldy];
    s += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += ws[w];
    part[blockIdx.x] = t;
  }
}

// S = [s X; t I]: the top m rows s X, the bottom n rows t times the identity.
__global__ void stack_kernel(int m, int n, const float* __restrict__ X, int64_t ldx, float s, float t, float* S,
                             int64_t lds) {
  const int64_t total = static_cast<int64_t>(m + n) * n;
  for (int64_t e = blockIdx.x * 256LL + threadIdx.x; e < total; e += 256LL * gridDim.x) {
    const int64_t j = e / (m + n), i = e - j * (m + n);
    float v;
    if (i < m)
      v = s * X[i + j * ldx];
    else
      v = (i - m == j) ? t : 0.f;
    S[i + j * lds] = v;
  }
}

// Y = alpha X (m x n)
__global__ void scale_copy_kernel(int m, int n, float alpha, const float* __restrict__ X, int64_t ldx, float* Y,
                                  int64_t ldy) {
  const int64_t total = static_cast<int64_t>(m) * n;
  for (int64_t e = blockIdx.x * 256LL + threadIdx.x; e < total; e += 256LL * gridDim.x) {
    const int64_t j = e / m, i = e - j * m;
    Y[i + j * ldy] = alpha * X[i + j * ldx];
  }
}

// Y = (X + X^T) / 2 (n x n, out of place); with transpose_upper, the
// transpose of an upper-triangular X into a lower-triangular Y instead
// (Y[i][j] = X[j][i] for i >= j, 0 above).
__global__ void sym_kernel(int n, const float* __restrict__ X, int64_t ldx, float* Y, int64_t ldy, int transpose_upper) {
  const int64_t total = static_cast<int64_t>(n) * n;
  for (int64_t e = blockIdx.x * 256LL + threadIdx.x; e < total; e += 256LL * gridDim.x) {
    const int64_t j = e / n, i = e - j * n;
    float v;
    if (transpose_upper)
      v = i >= j ? X[j + i * ldx] : 0.f;
    else
      v = 0.5f * (X[i + j * ldx] + X[j + i * ldx]);
    Y[i + j * ldy] = v;
  }
}

__global__ void eye_kernel(int n, float* Y, int64_t ldy) {
  const int64_t total = static_cast<int64_t>(n) * n;
  for (int64_t e = blockIdx.x * 256LL + threadIdx.x; e < total; e += 256LL * gridDim.x) {
    const int64_t j = e / n, i = e - j * n;
    Y[i + j * ldy] = i == j ? 1.f : 0.f;
  }
}

int grid_for(int64_t total) { return static_cast<int>(std::min<int64_t>((total + 255) / 256, 152 * 16)); }

struct QLayout {
  float* S;      // (m + n) x n stack, then its Q
  int64_t lds;
  float* R;      // n x n
  float* Xn;     // m x n next iterate
  float* L;      // n x n lower (R0^T), then R0^{-1}
  float* Rinv;
  double* part;  // kNormBlocks
  char* q1h;     // 16-bit copies of Q1 (m x n) and Q2 (n x n); reused for U and A when forming H
  char* q1l;
  char* q2h;
  char* q2l;
  int64_t ldq1, ldq2;
  float* qr_work;
  int64_t qr_lwork;
  void* qr_hwork;
  int64_t qr_lhwork;
  float* tr_work;
  int64_t tr_lwork;
  void* tr_hwork;
  int64_t tr_lhwork;
};

Options qr_options(const Options& o) {
  Options q = o;
  q.cgs2 = 1;
  if (q.prec == LATER_PREC_SPLIT2) q.prec = LATER_PREC_SPLIT3;
  return q;
}

bool carve_qdwh(Arena& fw, Arena& hw, int m, int n, const Options& o, QLayout* L) {
  const Options q = qr_options(o);
  const bool split = q.prec == LATER_PREC_SPLIT3;
  L->lds = m + n;
  L->S = fw.take<float>(static_cast<size_t>(L->lds) * n);
  L->R = fw.take<float>(static_cast<size_t>(n) * n);
  L->Xn = fw.take<float>(static_cast<size_t>(m) * n);
  L->L = fw.take<float>(static_cast<size_t>(n) * n);
  L->Rinv = fw.take<float>(static_cast<size_t>(n) * n);
  L->part = fw.take<double>(kNormBlocks);
  const QrNeed qn = rgsqrf_need(m + n, n, q);
  L->qr_lwork = qn.rec_work;
  L->qr_work = fw.take<float>(qn.rec_work);
  Options t;
  t.prec = LATER_PREC_FP16;
  L->tr_lwork = splitk_work();
  L->tr_work = fw.take<float>(L->tr_lwork);
  L->ldq1 = round_up(m, 8);
  L->ldq2 = round_up(n, 8);
  L->q1h = reinterpret_cast<char*>(hw.take<uint16_t>(L->ldq1 * n));
  L->q1l = split ? reinterpret_cast<char*>(hw.take<uint16_t>(L->ldq1 * n)) : nullptr;
  L->q2h = reinterpret_cast<char*>(hw.take<uint16_t>(L->ldq2 * n));
  L->q2l = split ? reinterpret_cast<char*>(hw.take<uint16_t>(L->ldq2 * n)) : nullptr;
  L->qr_lhwork = qn.hwork;
  L->qr_hwork = hw.take<uint16_t>(qn.hwork);
  L->tr_lhwork = rtrsm_hwork(n, n, 'r', t);
  L->tr_hwork = hw.take<uint16_t>(L->tr_lhwork);
  return !fw.failed() && !hw.failed();
}

later_status_t frob2(cudaStream_t st, int m, int n, const float* X, int64_t ldx, const float* Y, int64_t ldy,
                     double* part, double* out) {
  sumsq_kernel<<<kNormBlocks, 256, 0, st>>>(m, n, X, ldx, Y, ldy, part);
  note_launch();
  LATER_CHECK_CUDA(cudaGetLastError());
  std::vector<double> h(kNormBlocks);
  LATER_CHECK_CUDA(cudaMemcpyAsync(h.data(), part, sizeof(double) * kNormBlocks, cudaMemcpyDeviceToHost, st));
  LATER_CHECK_CUDA(cudaStreamSynchronize(st));
  double s = 0.0;
  for (double v : h) s += v;  // fixed order: deterministic
  *out = s;
  return LATER_OK;
}

later_status_t gemm_tc(cudaStream_t st, const Options& o, char ta, char tb, int M, int N, int K, float alpha,
                       const char* ah, const char* al, int64_t lda16, const char* bh, const char* bl, int64_t ldb16,
                       float beta, const float* C, int64_t ldc, float* D, int64_t ldd, float* work, int64_t lwork) {
  Scratch sc;
  if (work && lwork > 8192) {
    sc.counters = reinterpret_cast<int*>(work);
    sc.n_counters = 4096;
    sc.partial = work + 4096;
    sc.partial_floats = lwork - 4096;
    LATER_CHECK_CUDA(cudaMemsetAsync(sc.counters, 0, 4096 * sizeof(int), st));
  }
  GemmCall g;
  g.ta = ta;
  g.tb = tb;
  g.M = M;
  g.N = N;
  g.K = K;
  g.A = Op16{ah, al, lda16};
  g.B = Op16{bh, bl, ldb16};
  g.alpha = alpha;
  g.beta = beta;
  g.out.C = C;
  g.out.ldc = ldc;
  g.out.D = D;
  g.out.ldd = ldd;
  g.prec = o.prec;
  g.out_prec = o.prec;
  return tc_gemm(g, sc, st, o.budget);
}

}  // namespace

QrNeed qdwh_need(int m, int n, const Options& o) {
  Arena fw(nullptr, 0), hw(nullptr, 0);
  QLayout L;
  carve_qdwh(fw, hw, m, n, o, &L);
  QrNeed q;
  q.min_work = q.rec_work = static_cast<int64_t>(fw.peak() / sizeof(float)) + 64;
  q.hwork = static_cast<int64_t>(hw.peak() / 2) + 128;
  return q;
}

later_status_t qdwh_polar(cudaStream_t st, int m, int n, const float* A, int64_t lda, float* U, int64_t ldu, float* H,
                          int64_t ldh, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o,
                          double l0, int symmetrize, double tol, int max_iter, int* iterations) {
  if (m < 1 || n < 1 || m < n || lda < m || ldu < m || !A || !U) return LATER_ERR_INVALID_ARG;
  if (H && ldh < n) return LATER_ERR_INVALID_ARG;
  if (symmetrize && m != n) return LATER_ERR_INVALID_ARG;
  if (o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT2) return LATER_ERR_INVALID_ARG;
  if (n % 32 != 0) return LATER_ERR_INVALID_ARG;  // rgsqrf's column granularity
  if (tol <= 0) tol = 1e-6;
  if (max_iter <= 0) max_iter = 10;
  const QrNeed need = qdwh_need(m, n, o);
  if (!work || !hwork || lwork < need.min_work || lhwork < need.hwork) return LATER_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(hwork) & 15) != 0) return LATER_ERR_INVALID_ARG;
  Arena fw(work, static_cast<size_t>(lwork) * sizeof(float));
  Arena hw(hwork, static_cast<size_t>(lhwork) * 2);
  QLayout L;
  if (!carve_qdwh(fw, hw, m, n, o, &L)) return LATER_ERR_WORKSPACE;
  const Options qo = qr_options(o);
  const int gp = qo.prec;  // precision of the GEMMs (FP16 / BF16 / SPLIT3)
  Options go = o;
  go.prec = gp;

  // X0 = A / ||A||_F in U
  double a2 = 0.0;
  LATER_CHECK(frob2(st, m, n, A, lda, nullptr, 0, L.part, &a2));
  if (!(a2 > 0.0) || !std::isfinite(a2)) return LATER_ERR_NUMERIC;
  const double alpha = std::sqrt(a2);
  scale_copy_kernel<<<grid_for(static_cast<int64_t>(m) * n), 256, 0, st>>>(m, n, static_cast<float>(1.0 / alpha), A,
                                                                           lda, U, ldu);
  note_launch();
  LATER_CHECK_CUDA(cudaGetLastError());

  // l0 <= sigma_min(X0): 1 / ||R0^{-1}||_F for X0 = Q0 R0
  double l = l0;
  if (!(l > 0.0)) {
    LATER_CHECK(copy2d(st, m, n, U, ldu, L.S, L.lds));
    LATER_CHECK(rgsqrf(st, m, n, L.S, L.lds, L.R, n, L.qr_work, L.qr_lwork, L.qr_hwork, L.qr_lhwork, qo));
    sym_kernel<<<grid_for(static_cast<int64_t>(n) * n), 256, 0, st>>>(n, L.R, n, L.L, n, 1);  // L = R0^T
    eye_kernel<<<grid_for(static_cast<int64_t>(n) * n), 256, 0, st>>>(n, L.Rinv, n);
    note_launch(2);
    LATER_CHECK_CUDA(cudaGetLastError());
    Options t;
    t.prec = LATER_PREC_FP16;
    t.budget = o.budget;
    // X L^T = I  =>  X = L^{-T} = R0^{-1}; FP32 throughout
    LATER_CHECK(rtrsm_lim(st, 'l', 'r', 't', n, n, L.L, n, L.Rinv, n, L.tr_work, L.tr_lwork, L.tr_hwork,
                          L.tr_lhwork, t, INT_MAX));
    double r2 = 0.0;
    LATER_CHECK(frob2(st, n, n, L.Rinv, n, nullptr, 0, L.part, &r2));
    if (!(r2 > 0.0) || !std::isfinite(r2)) return LATER_ERR_NUMERIC;
    l = 1.0 / std::sqrt(r2);
  }
  l = std::min(l, 1.0);

  const double tol1 = 10.0 * tol / 2.0, tol3 = std::cbrt(tol1);
  int it = 0;
  for (it = 1; it <= max_iter; ++it) {
    const double l2 = l * l;
    const double dd = std::cbrt(4.0 * (1.0 - l2) / (l2 * l2));
    const double sqd = std::sqrt(1.0 + dd);
    const double a = sqd + std::sqrt(8.0 - 4.0 * dd + 8.0 * (2.0 - l2) / (l2 * sqd)) / 2.0;
    const double b = (a - 1.0) * (a - 1.0) / 4.0;
    const double c = a + b - 1.0;
    l = std::min(1.0, l * (a + b * l2) / (1.0 + c * l2));
    // [sqrt(c) X; I] scaled by c^(-1/4): [c^(1/4) X; c^(-1/4) I]
    const double q4 = std::sqrt(std::sqrt(c));
    stack_kernel<<<grid_for(static_cast<int64_t>(m + n) * n), 256, 0, st>>>(m, n, U, ldu, static_cast<float>(q4),
                                                                           static_cast<float>(1.0 / q4), L.S, L.lds);
    note_launch();
    LATER_CHECK_CUDA(cudaGetLastError());
    LATER_CHECK(rgsqrf(st, m + n, n, L.S, L.lds, L.R, n, L.qr_work, L.qr_lwork, L.qr_hwork, L.qr_lhwork, qo));
    LATER_CHECK(convert16(st, m, n, L.S, L.lds, L.q1h, L.q1l, L.ldq1, gp));
    LATER_CHECK(convert16(st, n, n, L.S + m, L.lds, L.q2h, L.q2l, L.ldq2, gp));
    // X_new = (b/c) X + (a - b/c)/sqrt(c) Q1 Q2^T
    LATER_CHECK(gemm_tc(st, go, 'N', 'T', m, n, n, static_cast<float>((a - b / c) / std::sqrt(c)), L.q1h, L.q1l,
                        L.ldq1, L.q2h, L.q2l, L.ldq2, static_cast<float>(b / c), U, ldu, L.Xn, m, L.tr_work,
                        L.tr_lwork));
    float* Xn = L.Xn;
    if (symmetrize) {
      sym_kernel<<<grid_for(static_cast<int64_t>(n) * n), 256, 0, st>>>(n, L.Xn, m, L.Rinv, n, 0);
      note_launch();
      LATER_CHECK_CUDA(cudaGetLastError());
      Xn = L.Rinv;
    }
    double d2 = 0.0;
    LATER_CHECK(frob2(st, m, n, Xn, symmetrize ? n : m, U, ldu, L.part, &d2));
    LATER_CHECK(copy2d(st, m, n, Xn, symmetrize ? n : m, U, ldu));
    if (!std::isfinite(d2)) return LATER_ERR_NUMERIC;
    if (std::sqrt(d2) < tol3 && 1.0 - l < tol1) break;
  }
  if (iterations) *iterations = std::min(it, max_iter);
  if (H) {  // H = sym(U^T A)
    LATER_CHECK(convert16(st, m, n, U, ldu, L.q1h, L.q1l, L.ldq1, gp));
    char* ah = reinterpret_cast<char*>(L.qr_hwork);  // A's 16-bit copy in the QR scratch
    char* al = gp == LATER_PREC_SPLIT3 ? ah + L.ldq1 * n * 2 : nullptr;
    if (L.qr_lhwork < L.ldq1 * n * (al ? 2 : 1)) return LATER_ERR_WORKSPACE;
    LATER_CHECK(convert16(st, m, n, A, lda, ah, al, L.ldq1, gp));
    LATER_CHECK(gemm_tc(st, go, 'T', 'N', n, n, m, 1.f, L.q1h, L.q1l, L.ldq1, ah, al, L.ldq1, 0.f, nullptr, n, L.R,
                        n, L.tr_work, L.tr_lwork));
    sym_kernel<<<grid_for(static_cast<int64_t>(n) * n), 256, 0, st>>>(n, L.R, n, H, ldh, 0);
    note_launch();
    LATER_CHECK_CUDA(cudaGetLastError());
  }
  return LATER_OK;
}

}  // namespace later

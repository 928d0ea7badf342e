// extern "C" entry points (include/later_c.h). Argument checking and status
// mapping live here; the work is in the drivers.
#include <cuda_runtime.h>

#include "../../include/later_c.h"
#include "blas3.cuh"
#include "qr.cuh"
#include "runtime.cuh"
#include "solve.cuh"

using namespace later;

extern "C" {

void later_c_default_options(later_options_t* opt) {
  if (!opt) return;
  opt->precision = LATER_PREC_FP16;
  opt->cgs2 = 0;
  opt->leaf = 128;
  opt->panel = 0;
  opt->timeout_cycles = 0;
}

const char* later_c_status_string(later_status_t s) {
  switch (s) {
    case LATER_OK: return "ok";
    case LATER_ERR_INVALID_ARG: return "invalid argument";
    case LATER_ERR_WORKSPACE: return "workspace too small";
    case LATER_ERR_CUDA: return "CUDA runtime error";
    case LATER_ERR_TIMEOUT: return "device wait timed out";
    case LATER_ERR_NOT_SUPPORTED: return "not supported";
    case LATER_ERR_RANGE: return "value outside the FP16 operand range";
    case LATER_ERR_NUMERIC: return "non-positive pivot";
  }
  return "unknown status";
}

later_status_t later_c_device_status(later_stream_t stream) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (cudaStreamSynchronize(st) != cudaSuccess) return LATER_ERR_CUDA;
  int* p = device_status_ptr();
  if (!p) return LATER_ERR_CUDA;
  int v = 0;
  if (cudaMemcpy(&v, p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return LATER_ERR_CUDA;
  if (v != 0 && cudaMemset(p, 0, sizeof(int)) != cudaSuccess) return LATER_ERR_CUDA;
  if (v & DEV_TIMEOUT) return LATER_ERR_TIMEOUT;
  if (v & DEV_NUMERIC) return LATER_ERR_NUMERIC;
  if (v & DEV_RANGE) return LATER_ERR_RANGE;
  return LATER_OK;
}

later_status_t later_c_wait_selftest(later_stream_t stream, long long timeout_cycles) {
  if (timeout_cycles < 0) return LATER_ERR_INVALID_ARG;
  return wait_selftest(reinterpret_cast<cudaStream_t>(stream), timeout_cycles);
}

later_status_t later_c_rgsqrf_bufsize(int m, int n, const later_options_t* opt, int64_t* lwork, int64_t* lhwork) {
  if (m < 1 || n < 1 || m < n) return LATER_ERR_INVALID_ARG;
  const QrNeed q = rgsqrf_need(m, n, options_from(opt));
  if (lwork) *lwork = q.rec_work;
  if (lhwork) *lhwork = q.hwork;
  return LATER_OK;
}

later_status_t later_c_rgsqrf(later_stream_t stream, int m, int n, float* A, int lda, float* R, int ldr,
                              float* work, int64_t lwork, void* hwork, int64_t lhwork, const later_options_t* opt) {
  return rgsqrf(reinterpret_cast<cudaStream_t>(stream), m, n, A, lda, R, ldr, work, lwork, hwork, lhwork,
                options_from(opt));
}

later_status_t later_c_rgsqrf_host(later_stream_t stream, int m, int n, const float* hA, int ldha, float* hQ,
                                   int ldhq, float* hR, int ldhr, float* A, int lda, float* R, int ldr, float* work,
                                   int64_t lwork, void* hwork, int64_t lhwork, const later_options_t* opt) {
  return rgsqrf_host(reinterpret_cast<cudaStream_t>(stream), m, n, hA, ldha, hQ, ldhq, hR, ldhr, A, lda, R, ldr, work,
                     lwork, hwork, lhwork, options_from(opt));
}

later_status_t later_c_oc_rgsqrf_bufsize(int m, int panel, const later_options_t* opt, int64_t* dev_bytes) {
  if (m < 1 || panel < 32 || panel % 32 != 0) return LATER_ERR_INVALID_ARG;
  if (dev_bytes) *dev_bytes = oc_rgsqrf_bytes(m, panel, options_from(opt));
  return LATER_OK;
}

later_status_t later_c_oc_rgsqrf(later_stream_t stream, int m, int n, float* hA, int ldha, float* hR, int ldhr,
                                 int panel, void* dev, int64_t dev_bytes, const later_options_t* opt) {
  return oc_rgsqrf(reinterpret_cast<cudaStream_t>(stream), m, n, hA, ldha, hR, ldhr, panel, dev, dev_bytes,
                   options_from(opt));
}

later_status_t later_c_rhouqr_bufsize(int m, int n, const later_options_t* opt, int64_t* lwork, int64_t* lhwork) {
  if (m < 1 || n < 1 || m < n) return LATER_ERR_INVALID_ARG;
  const QrNeed q = rhouqr_need(m, n, options_from(opt));
  if (lwork) *lwork = q.rec_work;
  if (lhwork) *lhwork = q.hwork;
  return LATER_OK;
}

later_status_t later_c_bhouqr_bufsize(int m, int n, const later_options_t* opt, int64_t* lwork, int64_t* lhwork) {
  if (m < 1 || n < 1 || m < n) return LATER_ERR_INVALID_ARG;
  const QrNeed q = bhouqr_need(m, n, options_from(opt));
  if (lwork) *lwork = q.rec_work;
  if (lhwork) *lhwork = q.hwork;
  return LATER_OK;
}

later_status_t later_c_bhouqr(later_stream_t stream, int m, int n, float* A, int lda, float* W, int ldw, float* R,
                              int ldr, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                              const later_options_t* opt) {
  return bhouqr(reinterpret_cast<cudaStream_t>(stream), m, n, A, lda, W, ldw, R, ldr, work, lwork, hwork, lhwork,
                options_from(opt));
}

later_status_t later_c_qdwh_bufsize(int m, int n, const later_options_t* opt, int64_t* lwork, int64_t* lhwork) {
  if (m < 1 || n < 1 || m < n) return LATER_ERR_INVALID_ARG;
  const QrNeed q = qdwh_need(m, n, options_from(opt));
  if (lwork) *lwork = q.rec_work;
  if (lhwork) *lhwork = q.hwork;
  return LATER_OK;
}

later_status_t later_c_qdwh_polar(later_stream_t stream, int m, int n, const float* A, int lda, float* U, int ldu,
                                  float* H, int ldh, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                                  const later_options_t* opt, double l0, int symmetric, double tol, int max_iter,
                                  int* iterations) {
  return qdwh_polar(reinterpret_cast<cudaStream_t>(stream), m, n, A, lda, U, ldu, H, ldh, work, lwork, hwork, lhwork,
                    options_from(opt), l0, symmetric, tol, max_iter, iterations);
}

later_status_t later_c_sy2sb_bufsize(int n, int nb, const later_options_t* opt, int64_t* lwork, int64_t* lhwork) {
  if (n < 1 || nb < 1) return LATER_ERR_INVALID_ARG;
  const QrNeed q = sy2sb_need(n, nb, options_from(opt));
  if (lwork) *lwork = q.rec_work;
  if (lhwork) *lhwork = q.hwork;
  return LATER_OK;
}

later_status_t later_c_sy2sb(later_stream_t stream, int n, int nb, float* A, int lda, float* Y, int ldy, float* W,
                             int ldw, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                             const later_options_t* opt) {
  return sy2sb(reinterpret_cast<cudaStream_t>(stream), n, nb, A, lda, Y, ldy, W, ldw, work, lwork, hwork, lhwork,
               options_from(opt));
}

later_status_t later_c_rhouqr(later_stream_t stream, int m, int n, float* A, int lda, float* W, int ldw, float* R,
                              int ldr, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                              const later_options_t* opt) {
  return rhouqr(reinterpret_cast<cudaStream_t>(stream), m, n, A, lda, W, ldw, R, ldr, work, lwork, hwork, lhwork,
                options_from(opt));
}

later_status_t later_c_ormqr(later_stream_t stream, int m, int n, float* W, int ldw, const float* Y, int ldy,
                             float* work, int64_t lwork) {
  return ormqr(reinterpret_cast<cudaStream_t>(stream), m, n, W, ldw, Y, ldy, work, lwork);
}

later_status_t later_c_blas3_bufsize(char op, char side, int m, int n, const later_options_t* opt, int64_t* lwork,
                                     int64_t* lhwork) {
  const Options o = options_from(opt);
  if (m < 0 || n < 0 || o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT3) return LATER_ERR_INVALID_ARG;
  int64_t h = 0;
  switch (op | 0x20) {
    case 's': h = rsyrk_hwork(m, n, o); break;
    case 't': h = rtrsm_hwork(m, n, side, o); break;
    case 'm': h = rtrmm_hwork(m, n, o); break;
    case 'p': h = rpotrf_hwork(m, o); break;
    default: return LATER_ERR_INVALID_ARG;
  }
  if (lwork) *lwork = splitk_work();
  if (lhwork) *lhwork = h;
  return LATER_OK;
}

later_status_t later_c_rsyrk(later_stream_t stream, int n, int k, float alpha, const float* A, int lda, float beta,
                             float* C, int ldc, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                             const later_options_t* opt) {
  return rsyrk(reinterpret_cast<cudaStream_t>(stream), n, k, alpha, A, lda, beta, C, ldc, work, lwork, hwork, lhwork,
               options_from(opt));
}

later_status_t later_c_rtrsm(later_stream_t stream, char uplo, char leri, char trans, int m, int n, const float* A,
                             int lda, float* B, int ldb, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                             const later_options_t* opt) {
  return rtrsm(reinterpret_cast<cudaStream_t>(stream), uplo, leri, trans, m, n, A, lda, B, ldb, work, lwork, hwork,
               lhwork, options_from(opt));
}

later_status_t later_c_rtrmm(later_stream_t stream, int m, int n, const float* A, int lda, const float* B, int ldb,
                             float* C, int ldc, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                             const later_options_t* opt) {
  return rtrmm(reinterpret_cast<cudaStream_t>(stream), m, n, A, lda, B, ldb, C, ldc, work, lwork, hwork, lhwork,
               options_from(opt));
}

later_status_t later_c_rpotrf(later_stream_t stream, char uplo, int n, float* A, int lda, float* work,
                              int64_t lwork, void* hwork, int64_t lhwork, const later_options_t* opt) {
  return rpotrf(reinterpret_cast<cudaStream_t>(stream), uplo, n, A, lda, work, lwork, hwork, lhwork,
                options_from(opt));
}

later_status_t later_c_spd_solve_bufsize(int n, int nrhs, const later_options_t* opt, int64_t* lwork,
                                         int64_t* lhwork) {
  if (n < 1 || nrhs < 1) return LATER_ERR_INVALID_ARG;
  const SolveNeed s = spd_solve_need(n, nrhs, options_from(opt));
  if (lwork) *lwork = s.work;
  if (lhwork) *lhwork = s.hwork;
  return LATER_OK;
}

later_status_t later_c_spd_solve(later_stream_t stream, int n, int nrhs, const float* A, int lda, const float* B,
                                 int ldb, double* X, int ldx, float* work, int64_t lwork, void* hwork,
                                 int64_t lhwork, const later_options_t* opt, int max_iter, double tol,
                                 later_solve_info_t* info) {
  SolveInfo si;
  const later_status_t s = spd_solve(reinterpret_cast<cudaStream_t>(stream), n, nrhs, A, lda, B, ldb, X, ldx, work,
                                     lwork, hwork, lhwork, options_from(opt), max_iter, tol, &si);
  if (info) {
    info->iterations = si.iterations;
    info->factor_precision = si.factor_precision;
    info->backward_error = si.backward_error;
  }
  return s;
}

later_status_t later_c_ls_solve_bufsize(int m, int n, int nrhs, const later_options_t* opt, int64_t* lwork,
                                        int64_t* lhwork) {
  if (m < n || n < 1 || nrhs < 1) return LATER_ERR_INVALID_ARG;
  const SolveNeed s = ls_solve_need(m, n, nrhs, options_from(opt));
  if (lwork) *lwork = s.work;
  if (lhwork) *lhwork = s.hwork;
  return LATER_OK;
}

later_status_t later_c_ls_solve(later_stream_t stream, int m, int n, int nrhs, const float* A, int lda,
                                const float* B, int ldb, double* X, int ldx, float* work, int64_t lwork,
                                void* hwork, int64_t lhwork, const later_options_t* opt, int max_iter, double tol,
                                later_solve_info_t* info) {
  SolveInfo si;
  const later_status_t s = ls_solve(reinterpret_cast<cudaStream_t>(stream), m, n, nrhs, A, lda, B, ldb, X, ldx, work,
                                    lwork, hwork, lhwork, options_from(opt), max_iter, tol, &si);
  if (info) {
    info->iterations = si.iterations;
    info->factor_precision = si.factor_precision;
    info->backward_error = si.backward_error;
  }
  return s;
}

}  // extern "C"

namespace later {
int64_t batched_plan_bytes(int count);
later_status_t batched_plan(cudaStream_t st, int count, const later_qr_item_t* host_items, void* plan,
                            int64_t plan_bytes);
later_status_t batched_run(cudaStream_t st, int count, const void* plan, int* queue, int* status, int variant);
}  // namespace later

extern "C" {

int64_t later_c_batched_plan_bytes(int count) { return count > 0 ? batched_plan_bytes(count) : 0; }

later_status_t later_c_batched_qr_plan(later_stream_t stream, int count, const later_qr_item_t* items, void* plan,
                                       int64_t plan_bytes) {
  return batched_plan(reinterpret_cast<cudaStream_t>(stream), count, items, plan, plan_bytes);
}

later_status_t later_c_batched_qr_run(later_stream_t stream, int count, const void* plan, int* queue, int* status,
                                      int variant) {
  if (variant < -1 || variant > 3) return LATER_ERR_INVALID_ARG;
  return batched_run(reinterpret_cast<cudaStream_t>(stream), count, plan, queue, status, variant < 0 ? 0 : variant);
}

later_status_t later_c_gemm16(later_stream_t stream, char transa, char transb, int m, int n, int k, float alpha,
                              const void* A, int lda, const void* B, int ldb, float beta, const float* C, int ldc,
                              float* D, int ldd, int precision, float* work, int64_t lwork) {
  auto ok_t = [](char t) { return t == 'N' || t == 'n' || t == 'T' || t == 't'; };
  if (!ok_t(transa) || !ok_t(transb) || m < 0 || n < 0 || k < 1 || !A || !B || !D) return LATER_ERR_INVALID_ARG;
  if (precision != LATER_PREC_FP16 && precision != LATER_PREC_BF16) return LATER_ERR_INVALID_ARG;
  const bool an = (transa == 'N' || transa == 'n');
  const bool bn = (transb == 'N' || transb == 'n');
  if (lda < (an ? m : k) || ldb < (bn ? k : n) || ldd < m || (beta != 0.f && (!C || ldc < m)))
    return LATER_ERR_INVALID_ARG;
  GemmCall g;
  g.ta = transa;
  g.tb = transb;
  g.M = m;
  g.N = n;
  g.K = k;
  g.A = Op16{A, nullptr, lda};
  g.B = Op16{B, nullptr, ldb};
  g.alpha = alpha;
  g.beta = beta;
  g.out.C = C;
  g.out.ldc = ldc;
  g.out.D = D;
  g.out.ldd = ldd;
  g.prec = precision;
  Scratch s;
  if (work && lwork > 4096 * 2) {
    s.counters = reinterpret_cast<int*>(work);
    s.n_counters = 4096;
    s.partial = work + 4096;
    s.partial_floats = lwork - 4096;
    if (cudaMemsetAsync(s.counters, 0, 4096 * sizeof(int), reinterpret_cast<cudaStream_t>(stream)) != cudaSuccess)
      return LATER_ERR_CUDA;
  }
  return tc_gemm(g, s, reinterpret_cast<cudaStream_t>(stream), 0);
}

later_status_t later_c_convert(later_stream_t stream, int m, int n, const float* A, int lda, void* hi, void* lo,
                               int ldh, int precision) {
  if (m < 0 || n < 0 || !A || !hi || lda < m || ldh < m) return LATER_ERR_INVALID_ARG;
  if (precision < LATER_PREC_FP16 || precision > LATER_PREC_SPLIT3) return LATER_ERR_INVALID_ARG;
  return convert16(reinterpret_cast<cudaStream_t>(stream), m, n, A, lda, hi, lo, ldh, precision);
}

}  // extern "C"

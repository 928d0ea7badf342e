// C++-linkage drop-in entry points of include/LATER.h, on top of the C ABI.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <utility>

#include "../../include/LATER.h"
#include "blas3.cuh"
#include "qr.cuh"

namespace {

thread_local later_status_t g_last = LATER_OK;

later_status_t record(const char* fn, later_status_t s) {
  g_last = s;
  if (s != LATER_OK) std::fprintf(stderr, "%s: %s\n", fn, later_c_status_string(s));
  return s;
}

// Stream of a cuBLAS handle when cuBLAS is loaded in the process (looked up at
// run time; the library itself does not link cuBLAS), else the default stream.
cudaStream_t stream_of(cublasHandle_t h) {
  if (!h) return nullptr;
  using Fn = cublasStatus_t (*)(cublasHandle_t, cudaStream_t*);
  static Fn fn = reinterpret_cast<Fn>(dlsym(RTLD_DEFAULT, "cublasGetStream_v2"));
  cudaStream_t s = nullptr;
  if (fn && fn(h, &s) == CUBLAS_STATUS_SUCCESS) return s;
  return nullptr;
}

// Library-owned workspace for the routines whose reference signatures carry
// no workspace (rtrsm, rsyrk, rtrmm, rpotrf) or too little (bhouqr): one float and one 16-bit buffer
// per (device, stream), grown to the largest request seen on that stream and
// kept until exit. A call holds the cache lock from the lookup until its work
// is enqueued, so each buffer is used in its stream's order only: calls on
// different streams (or host threads with different cuBLAS-handle streams)
// get different buffers, and a buffer that grows is released with
// cudaFreeAsync on its own stream, after the work already queued there.
struct Entry {
  float* work = nullptr;
  size_t lwork = 0;
  void* hwork = nullptr;
  size_t lhwork = 0;
};
struct Cache {
  std::mutex mu;
  std::map<std::pair<int, cudaStream_t>, Entry> entries;
};
Cache& cache() {
  static Cache c;
  return c;
}

template <class Fn>
later_status_t with_workspace(cudaStream_t st, int64_t lw, int64_t lh, Fn fn) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return LATER_ERR_CUDA;
  Cache& c = cache();
  std::lock_guard<std::mutex> g(c.mu);
  Entry& e = c.entries[{dev, st}];
  if (static_cast<size_t>(lw) > e.lwork) {
    if (e.work && cudaFreeAsync(e.work, st) != cudaSuccess) return LATER_ERR_CUDA;
    e.work = nullptr;
    e.lwork = 0;
    if (cudaMallocAsync(reinterpret_cast<void**>(&e.work), static_cast<size_t>(lw) * sizeof(float), st) !=
        cudaSuccess)
      return LATER_ERR_CUDA;
    e.lwork = static_cast<size_t>(lw);
  }
  if (static_cast<size_t>(lh) > e.lhwork) {
    if (e.hwork && cudaFreeAsync(e.hwork, st) != cudaSuccess) return LATER_ERR_CUDA;
    e.hwork = nullptr;
    e.lhwork = 0;
    if (cudaMallocAsync(&e.hwork, static_cast<size_t>(lh) * 2, st) != cudaSuccess) return LATER_ERR_CUDA;
    e.lhwork = static_cast<size_t>(lh);
  }
  return fn(e.work, static_cast<int64_t>(e.lwork), e.hwork, static_cast<int64_t>(e.lhwork));
}

}  // namespace

using namespace later;

void later_rgsqrf(cudaCtxt ctxt, int m, int n, float* A, int lda, float* R, int ldr, float* work, int lwork,
                  __half* hwork, int lhwork) {
  record("later_rgsqrf", rgsqrf(stream_of(ctxt.cublas_handle), m, n, A, lda, R, ldr, work, lwork, hwork, lhwork,
                                Options{}));
}

void later_rhouqr(cudaCtxt ctxt, int m, int n, float* A, int lda, float* W, int ldw, float* R, int ldr, float* work,
                  int lwork, __half* hwork, int lhwork, float* /*U: not needed*/) {
  record("later_rhouqr", rhouqr(stream_of(ctxt.cublas_handle), m, n, A, lda, W, ldw, R, ldr, work, lwork, hwork,
                                lhwork, Options{}));
}

void later_ormqr(int m, int n, float* W, int ldw, float* Y, int ldy, float* work) {
  // The caller's work holds m*n floats (QR/later_ormqr.cu:48 allocated that much itself).
  record("later_ormqr", ormqr(nullptr, m, n, W, ldw, Y, ldy, work, static_cast<int64_t>(m) * n));
}

void later_bhouqr(int m, int n, float* A, int lda, float* W, int ldw, float* R, int ldr, float*, int, __half*, int,
                  float* /*U: not needed*/) {
  Options o;
  o.prec = LATER_PREC_SPLIT3;  // the reference's updates are FP32 SGEMMs (QR/later_bhouqr.cu:122-165)
  const QrNeed q = bhouqr_need(m, n, o);
  record("later_bhouqr", with_workspace(nullptr, q.rec_work, q.hwork, [&](float* w, int64_t lw, void* h, int64_t lh) {
           return bhouqr(nullptr, m, n, A, lda, W, ldw, R, ldr, w, lw, h, lh, o);
         }));
}

void later_qdwh_polar(cudaCtxt ctxt, int n, float* A, int lda, float* H, int ldh, float* tmpA, float*, __half*) {
  Options o;
  o.prec = LATER_PREC_SPLIT3;
  cudaStream_t st = stream_of(ctxt.cublas_handle);
  const QrNeed q = qdwh_need(n, n, o);
  record("later_qdwh_polar", with_workspace(st, q.rec_work, q.hwork, [&](float* w, int64_t lw, void* h, int64_t lh) {
           return qdwh_polar(st, n, n, tmpA, n, A, lda, H, ldh, w, lw, h, lh, o, 0.0, 1, 1e-6, 10, nullptr);
         }));
}

void later_sy2sb_rec(cudaCtxt ctxt, int n, int /*ns*/, float* A, float* /*oriA*/, int lda, float*, int, __half*, int) {
  Options o;
  o.prec = LATER_PREC_SPLIT3;
  cudaStream_t st = stream_of(ctxt.cublas_handle);
  const QrNeed q = sy2sb_need(n, 128, o);
  record("later_sy2sb_rec", with_workspace(st, q.rec_work, q.hwork, [&](float* w, int64_t lw, void* h, int64_t lh) {
           return sy2sb(st, n, 128, A, lda, nullptr, 0, nullptr, 0, w, lw, h, lh, o);
         }));
}

void ssytrd_sy2sb(cudaCtxt ctxt, int n, int nb, float* A, float* A_cpy, int lda, float*, int, __half*, int) {
  Options o;
  o.prec = LATER_PREC_SPLIT3;
  cudaStream_t st = stream_of(ctxt.cublas_handle);
  const QrNeed q = sy2sb_need(n, nb, o);
  record("ssytrd_sy2sb", with_workspace(st, q.rec_work, q.hwork, [&](float* w, int64_t lw, void* h, int64_t lh) {
           return sy2sb(st, n, nb, A_cpy, lda, A, lda, nullptr, 0, w, lw, h, lh, o);
         }));
}

void later_ormqr2(int m, int n, float* W, int ldw, float* Y, int ldy, float* work) {
  record("later_ormqr2", ormqr(nullptr, m, n, W, ldw, Y, ldy, work, static_cast<int64_t>(m) * n));
}

void later_rtrsm(cublasHandle_t handle, char uplo, char leri, char trans, int m, int n, float* A, int lda, float* B,
                 int ldb, __half*) {
  const Options o;
  cudaStream_t st = stream_of(handle);
  record("later_rtrsm", with_workspace(st, splitk_work(), rtrsm_hwork(m, n, leri, o),
                                       [&](float* w, int64_t lw, void* h, int64_t lh) {
                                         return rtrsm(st, uplo, leri, trans, m, n, A, lda, B, ldb, w, lw, h, lh, o);
                                       }));
}

void later_rsyrk(cublasHandle_t handle, int n, int k, float alpha, float* A, int lda, float beta, float* C, int ldc,
                 __half*) {
  const Options o;
  cudaStream_t st = stream_of(handle);
  record("later_rsyrk", with_workspace(st, splitk_work(), rsyrk_hwork(n, k, o),
                                       [&](float* w, int64_t lw, void* h, int64_t lh) {
                                         return rsyrk(st, n, k, alpha, A, lda, beta, C, ldc, w, lw, h, lh, o);
                                       }));
}

void later_rtrmm(int m, int n, float* A, int lda, float* B, int ldb, float* C, int ldc, float* /*tempC*/, __half*) {
  const Options o;
  record("later_rtrmm", with_workspace(nullptr, splitk_work(), rtrmm_hwork(m, n, o),
                                       [&](float* w, int64_t lw, void* h, int64_t lh) {
                                         return rtrmm(nullptr, m, n, A, lda, B, ldb, C, ldc, w, lw, h, lh, o);
                                       }));
}

void later_rpotrf(char uplo, int n, float* A, int lda, float*, __half*) {
  const Options o;
  record("later_rpotrf", with_workspace(nullptr, splitk_work(), rpotrf_hwork(n, o),
                                        [&](float* w, int64_t lw, void* h, int64_t lh) {
                                          return rpotrf(nullptr, uplo, n, A, lda, w, lw, h, lh, o);
                                        }));
}

later_status_t later_get_last_status() { return g_last; }

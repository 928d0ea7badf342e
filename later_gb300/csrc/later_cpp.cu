// C++-linkage drop-in entry points of include/LATER.h, on top of the C ABI.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

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
// no workspace sizes: one float and one 16-bit buffer per device, grown to the
// largest request seen, kept until exit.
struct Cache {
  std::mutex mu;
  float* work[64] = {};
  size_t lwork[64] = {};
  void* hwork[64] = {};
  size_t lhwork[64] = {};
};
Cache& cache() {
  static Cache c;
  return c;
}

later_status_t cached(int64_t lw, int64_t lh, float** work, void** hwork) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return LATER_ERR_CUDA;
  Cache& c = cache();
  std::lock_guard<std::mutex> g(c.mu);
  if (static_cast<size_t>(lw) > c.lwork[dev]) {
    cudaDeviceSynchronize();
    if (c.work[dev]) cudaFree(c.work[dev]);
    c.work[dev] = nullptr;
    c.lwork[dev] = 0;
    if (cudaMalloc(&c.work[dev], static_cast<size_t>(lw) * sizeof(float)) != cudaSuccess) return LATER_ERR_CUDA;
    c.lwork[dev] = static_cast<size_t>(lw);
  }
  if (static_cast<size_t>(lh) > c.lhwork[dev]) {
    cudaDeviceSynchronize();
    if (c.hwork[dev]) cudaFree(c.hwork[dev]);
    c.hwork[dev] = nullptr;
    c.lhwork[dev] = 0;
    if (cudaMalloc(&c.hwork[dev], static_cast<size_t>(lh) * 2) != cudaSuccess) return LATER_ERR_CUDA;
    c.lhwork[dev] = static_cast<size_t>(lh);
  }
  *work = c.work[dev];
  *hwork = c.hwork[dev];
  return LATER_OK;
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

void later_ormqr2(int m, int n, float* W, int ldw, float* Y, int ldy, float* work) {
  record("later_ormqr2", ormqr(nullptr, m, n, W, ldw, Y, ldy, work, static_cast<int64_t>(m) * n));
}

void later_rtrsm(cublasHandle_t handle, char uplo, char leri, char trans, int m, int n, float* A, int lda, float* B,
                 int ldb, __half*) {
  const Options o;
  float* w = nullptr;
  void* h = nullptr;
  const int64_t lh = rtrsm_hwork(m, n, leri, o), lw = splitk_work();
  later_status_t s = cached(lw, lh, &w, &h);
  if (s == LATER_OK) s = rtrsm(stream_of(handle), uplo, leri, trans, m, n, A, lda, B, ldb, w, lw, h, lh, o);
  record("later_rtrsm", s);
}

void later_rsyrk(cublasHandle_t handle, int n, int k, float alpha, float* A, int lda, float beta, float* C, int ldc,
                 __half*) {
  const Options o;
  float* w = nullptr;
  void* h = nullptr;
  const int64_t lh = rsyrk_hwork(n, k, o), lw = splitk_work();
  later_status_t s = cached(lw, lh, &w, &h);
  if (s == LATER_OK) s = rsyrk(stream_of(handle), n, k, alpha, A, lda, beta, C, ldc, w, lw, h, lh, o);
  record("later_rsyrk", s);
}

void later_rtrmm(int m, int n, float* A, int lda, float* B, int ldb, float* C, int ldc, float* /*tempC*/, __half*) {
  const Options o;
  float* w = nullptr;
  void* h = nullptr;
  const int64_t lh = rtrmm_hwork(m, n, o), lw = splitk_work();
  later_status_t s = cached(lw, lh, &w, &h);
  if (s == LATER_OK) s = rtrmm(nullptr, m, n, A, lda, B, ldb, C, ldc, w, lw, h, lh, o);
  record("later_rtrmm", s);
}

void later_rpotrf(char uplo, int n, float* A, int lda, float*, __half*) {
  const Options o;
  float* w = nullptr;
  void* h = nullptr;
  const int64_t lh = rpotrf_hwork(n, o), lw = splitk_work();
  later_status_t s = cached(lw, lh, &w, &h);
  if (s == LATER_OK) s = rpotrf(nullptr, uplo, n, A, lda, w, lw, h, lh, o);
  record("later_rpotrf", s);
}

later_status_t later_get_last_status() { return g_last; }

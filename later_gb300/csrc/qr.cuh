// Recursive QR drivers (host side): rgsqrf now, rhouqr / ormqr alongside.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "runtime.cuh"

namespace later {

struct Options {
  int prec = LATER_PREC_FP16;
  int cgs2 = 0;
  int leaf = 128;
  int panel = 0;  // 0: fused leaf, 32-column CholQR2 panels; 2: fused, leaf-wide CholQR2 first; 1: MGS-TSQR
  long long budget = kDefaultBudgetCycles;
};

Options options_from(const later_options_t* o);

// Workspace need of later_c_rgsqrf: `min_*` is what the call refuses to run
// below, `rec_*` what the *_bufsize query reports (adds room for split-K and
// for fully parallel panel projections).
struct QrNeed {
  int64_t min_work = 0, rec_work = 0;  // floats
  int64_t hwork = 0;                   // 16-bit elements
};
QrNeed rgsqrf_need(int m, int n, const Options& o);

later_status_t rgsqrf(cudaStream_t st, int m, int n, float* A, int64_t lda, float* R, int64_t ldr, float* work,
                      int64_t lwork, void* hwork, int64_t lhwork, const Options& o);

// rgsqrf on host buffers: hA is copied in and Q, R copied out in column
// chunks on two copy streams overlapped with the factorisation (A, R are the
// device buffers it runs in); `st` completes after the last copy.
later_status_t rgsqrf_host(cudaStream_t st, int m, int n, const float* hA, int64_t ldha, float* hQ, int64_t ldhq,
                           float* hR, int64_t ldhr, float* A, int64_t lda, float* R, int64_t ldr, float* work,
                           int64_t lwork, void* hwork, int64_t lhwork, const Options& o);

// Out-of-core rgsqrf through a caller-given device region (oc.cu).
int64_t oc_rgsqrf_bytes(int m, int panel, const Options& o);
later_status_t oc_rgsqrf(cudaStream_t st, int m, int n, float* hA, int64_t ldha, float* hR, int64_t ldhr, int panel,
                         void* dev, int64_t dev_bytes, const Options& o);

QrNeed rhouqr_need(int m, int n, const Options& o);

later_status_t rhouqr(cudaStream_t st, int m, int n, float* A, int64_t lda, float* W, int64_t ldw, float* R,
                      int64_t ldr, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o);

// Blocked Householder QR over 128-column rhouqr panels (QR/later_bhouqr.cu:88-189).
QrNeed bhouqr_need(int m, int n, const Options& o);
later_status_t bhouqr(cudaStream_t st, int m, int n, float* A, int64_t lda, float* W, int64_t ldw, float* R,
                      int64_t ldr, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o);

// QDWH polar decomposition A = U H (EVD/later_qdwh_polar.cu:24-110), qdwh.cu.
QrNeed qdwh_need(int m, int n, const Options& o);
later_status_t qdwh_polar(cudaStream_t st, int m, int n, const float* A, int64_t lda, float* U, int64_t ldu, float* H,
                          int64_t ldh, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o,
                          double l0, int symmetrize, double tol, int max_iter, int* iterations);

// Symmetric to band reduction B = Q^T A Q, bandwidth nb (sy2sb.cu).
QrNeed sy2sb_need(int n, int nb, const Options& o);
later_status_t sy2sb(cudaStream_t st, int n, int nb, float* A, int64_t lda, float* Y, int64_t ldy, float* W,
                     int64_t ldw, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o);

// Q = I - W Y^T (first n columns) written over W; `work` holds m x n floats.
later_status_t ormqr(cudaStream_t st, int m, int n, float* W, int64_t ldw, const float* Y, int64_t ldy, float* work,
                     int64_t lwork);

// Split point of a width-n recursion step: the larger half, in 32-column units.
inline int split_half(int n) { return ((n / 32 + 1) / 2) * 32; }

}  // namespace later

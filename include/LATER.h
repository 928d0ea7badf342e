/*
 * LATER.h — drop-in C++ header for the recursive QR / Cholesky hot path.
 *
 * Same declarations (C++ linkage, same parameter types) as the reference's
 * include/LATER.h for the routines this library implements, so a program
 * written against LATER (e.g. its test/test_qr.cu call sites) compiles and
 * links against liblater_gb300.so unchanged for these calls:
 *
 *   later_rgsqrf  LATER.h:39     later_rhouqr  LATER.h:41
 *   later_ormqr   LATER.h:43     later_bhouqr  LATER.h:45
 *   later_ormqr2  LATER.h:47
 *   later_rtrsm   LATER.h:60     later_rsyrk   LATER.h:62
 *   later_rtrmm   LATER.h:64     later_qdwh_polar LATER.h:70
 *   later_sy2sb_rec LATER.h:72   ssytrd_sy2sb  LATER.h:74
 *   later_rpotrf  LATER.h:80
 *
 * Behaviour differences (a superset of the reference's):
 *   - errors never exit(): every call records a later_status_t, readable with
 *     later_get_last_status(), and prints one line to stderr when not OK;
 *   - work runs on the stream of ctxt.cublas_handle / handle when the process
 *     has cuBLAS loaded (cublasGetStream is looked up at run time; this library
 *     does not link cuBLAS), else on the default stream;
 *   - any lda >= m is honoured; R is written in full, zeros below the diagonal;
 *   - later_qdwh_polar reads the n x n input from tmpA (ld n) and writes U to
 *     the top n x n block of A (lda >= n) and H to H, like the reference's
 *     (which leaves H untouched); it symmetrises every iterate as the
 *     reference does, so A must be symmetric; SPLIT3 + CGS2 QR, tolerance
 *     1e-6, library-owned workspace;
 *   - later_sy2sb_rec reduces the symmetric A (both triangles stored, lda)
 *     to band form in place with bandwidth 128 (ns, oriA unused);
 *     ssytrd_sy2sb reduces A_cpy in place with bandwidth nb and writes the
 *     reflectors Y below the band into A (the reference factors its panels
 *     from A while updating A_cpy). Both run in SPLIT3 with library-owned
 *     workspace; n must be a multiple of the bandwidth;
 *   - later_bhouqr runs its updates in SPLIT3 (the FP32 level of the
 *     reference's SGEMMs) and needs more scratch than the m*n work / hwork the
 *     reference's test passes; it uses the library-owned workspace below;
 *   - rtrsm / rsyrk / rtrmm / rpotrf, whose reference signatures carry no
 *     workspace sizes, use a library-owned workspace per (device, stream)
 *     instead of the caller's `work` / `hwork`. It grows when a larger
 *     problem arrives on that stream (cudaMallocAsync / cudaFreeAsync on the
 *     same stream, so no device-wide synchronisation) and is kept until exit.
 *     Calls from several host threads are safe: each stream has its own
 *     buffers, and calls on one stream use them in stream order. The C ABI
 *     (later_c.h) takes explicit workspaces and never allocates.
 * The helper functions of the reference header (timers, generators, s2h and
 * friends) and the out-of-core QR routines are not declared here.
 */
#pragma once

#include <cublas_v2.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include "later_c.h"

struct cudaCtxt {
  cublasHandle_t cublas_handle;
  cusolverDnHandle_t cusolver_handle;
};

void later_rgsqrf(cudaCtxt ctxt, int m, int n, float* A, int lda, float* R, int ldr, float* work, int lwork,
                  __half* hwork, int lhwork);

void later_rhouqr(cudaCtxt ctxt, int m, int n, float* A, int lda, float* W, int ldw, float* R, int ldr, float* work,
                  int lwork, __half* hwork, int lhwork, float* U);

void later_ormqr(int m, int n, float* W, int ldw, float* Y, int ldy, float* work);

void later_bhouqr(int m, int n, float* A, int lda, float* W, int ldw, float* R, int ldr, float* work, int lwork,
                  __half* hwork, int lhwork, float* U);

void later_ormqr2(int m, int n, float* W, int ldw, float* Y, int ldy, float* work);

void later_rtrsm(cublasHandle_t handle, char uplo, char leri, char trans, int m, int n, float* A, int lda, float* B,
                 int ldb, __half* work);

void later_rsyrk(cublasHandle_t handle, int n, int k, float alpha, float* A, int lda, float beta, float* C, int ldc,
                 __half* work);

void later_rtrmm(int m, int n, float* A, int lda, float* B, int ldb, float* C, int ldc, float* tempC, __half* hwork);

void later_rpotrf(char uplo, int n, float* A, int lda, float* work, __half* hwork);

void later_qdwh_polar(cudaCtxt ctxt, int n, float* A, int lda, float* H, int ldh, float* tmpA, float* work,
                      __half* hwork);

void later_sy2sb_rec(cudaCtxt ctxt, int n, int ns, float* A, float* oriA, int lda, float* work, int lwork,
                     __half* hwork, int lhwork);

void ssytrd_sy2sb(cudaCtxt ctxt, int n, int nb, float* A, float* A_cpy, int lda, float* work, int lwork,
                  __half* hwork, int lhwork);

/* Status of the last call made through this header on the calling thread. */
later_status_t later_get_last_status();

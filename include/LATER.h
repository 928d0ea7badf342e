/*
 * LATER.h — drop-in C++ header for the recursive QR / Cholesky hot path.
 *
 * Same declarations (C++ linkage, same parameter types) as the reference's
 * include/LATER.h for the routines this library implements, so a program
 * written against LATER (e.g. its test/test_qr.cu call sites) compiles and
 * links against liblater_gb300.so unchanged for these calls:
 *
 *   later_rgsqrf  LATER.h:39     later_rhouqr  LATER.h:41
 *   later_ormqr   LATER.h:43     later_ormqr2  LATER.h:47
 *   later_rtrsm   LATER.h:60     later_rsyrk   LATER.h:62
 *   later_rtrmm   LATER.h:64     later_rpotrf  LATER.h:80
 *
 * Behaviour differences (a superset of the reference's):
 *   - errors never exit(): every call records a later_status_t, readable with
 *     later_get_last_status(), and prints one line to stderr when not OK;
 *   - work runs on the stream of ctxt.cublas_handle / handle when the process
 *     has cuBLAS loaded (cublasGetStream is looked up at run time; this library
 *     does not link cuBLAS), else on the default stream;
 *   - any lda >= m is honoured; R is written in full, zeros below the diagonal;
 *   - rtrsm / rsyrk / rtrmm / rpotrf, whose reference signatures carry no
 *     workspace sizes, use a library-owned workspace per (device, stream)
 *     instead of the caller's `work` / `hwork`. It grows when a larger
 *     problem arrives on that stream (cudaMallocAsync / cudaFreeAsync on the
 *     same stream, so no device-wide synchronisation) and is kept until exit.
 *     Calls from several host threads are safe: each stream has its own
 *     buffers, and calls on one stream use them in stream order. The C ABI
 *     (later_c.h) takes explicit workspaces and never allocates.
 * The helper functions of the reference header (timers, generators, s2h and
 * friends, the out-of-core / EVD / blocked routines) are outside this
 * library's scope and are not declared here.
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

void later_ormqr2(int m, int n, float* W, int ldw, float* Y, int ldy, float* work);

void later_rtrsm(cublasHandle_t handle, char uplo, char leri, char trans, int m, int n, float* A, int lda, float* B,
                 int ldb, __half* work);

void later_rsyrk(cublasHandle_t handle, int n, int k, float alpha, float* A, int lda, float beta, float* C, int ldc,
                 __half* work);

void later_rtrmm(int m, int n, float* A, int lda, float* B, int ldb, float* C, int ldc, float* tempC, __half* hwork);

void later_rpotrf(char uplo, int n, float* A, int lda, float* work, __half* hwork);

/* Status of the last call made through this header on the calling thread. */
later_status_t later_get_last_status();

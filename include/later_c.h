/*
 * later_c.h — C ABI of the GB300 (sm_103a) recursive QR / Cholesky library.
 *
 * Every entry point takes plain device pointers, sizes and leading dimensions
 * (column-major, element (i,j) at A[i + j*lda]), runs asynchronously on the
 * given CUDA stream and returns a later_status_t for argument / launch errors.
 * Failures detected on the device (a bounded wait that gave up, an FP16 range
 * overflow, a non-positive Cholesky pivot) are collected in a per-device
 * status word; later_c_device_status() synchronises and returns it.
 *
 * Buffers follow the reference interface (include/LATER.h of LATER): the
 * caller owns A, R, W and two workspaces — `work` (float) and `hwork` (16-bit)
 * — whose minimum sizes the *_bufsize queries return. Nothing on these paths
 * allocates device memory.
 */
#ifndef LATER_C_H
#define LATER_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* later_stream_t; /* same type as cudaStream_t */

typedef enum {
  LATER_OK = 0,
  LATER_ERR_INVALID_ARG = 1, /* bad size / leading dimension / flag */
  LATER_ERR_WORKSPACE = 2,   /* work or hwork smaller than the *_bufsize query */
  LATER_ERR_CUDA = 3,        /* a CUDA runtime call or launch failed */
  LATER_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
  LATER_ERR_NOT_SUPPORTED = 5,
  LATER_ERR_RANGE = 6,       /* a value exceeded the FP16 operand range: use BF16 */
  LATER_ERR_NUMERIC = 7      /* non-positive pivot (matrix not SPD) */
} later_status_t;

typedef enum {
  LATER_PREC_FP16 = 0,  /* FP16 tensor-core products, FP32 accumulation (reference behaviour) */
  LATER_PREC_BF16 = 1,  /* BF16 products, FP32 accumulation (range-safe) */
  LATER_PREC_SPLIT3 = 2, /* hi+lo FP16 split, three products per GEMM: ~FP32 accuracy */
  LATER_PREC_SPLIT2 = 3  /* rgsqrf (and the LS solver) only: R12 = Q1^T A2 as one FP16 product kept at its
                            FP16 value, A2 -= Q1 R12 with Q1 split hi+lo (two products): backward error at
                            the FP32 level, orthogonality as FP16, 1.5x the FP16 tensor work */
} later_precision_t;

typedef struct {
  int precision;            /* later_precision_t for every tensor-core GEMM */
  int cgs2;                 /* 1: second Gram-Schmidt pass in every panel (CGS2) */
  int leaf;                 /* rgsqrf leaf width: 32, 64 or 128 (0 = 128, the reference's NMIN) */
  int panel;                /* rgsqrf leaf: 0 = one fused launch per leaf, CholQR2 per 32-column
                               panel with an MGS-TSQR fallback (default); 2 = the fused launch
                               first trying one CholQR2 over the whole leaf (better orthogonality,
                               slower today), else as 0; 1 = MGS-TSQR panels and separate
                               block-CGS launches (the reference's algorithm) */
  long long timeout_cycles; /* bound on every device wait in SM cycles (0 = about one second) */
} later_options_t;

/* Fills the defaults: FP16, no CGS2, leaf 128, default timeout. */
void later_c_default_options(later_options_t* opt);

const char* later_c_status_string(later_status_t s);

/* Synchronises `stream`, then returns and clears the device status word. */
later_status_t later_c_device_status(later_stream_t stream);

/*
 * Failure-detection self-check (no counterpart in the reference, which has no
 * bounded waits): enqueues one small kernel whose two device waits, on an
 * mbarrier phase and on a global flag that nothing ever completes, give up
 * after `timeout_cycles` SM cycles (0 = the default of about one second). The
 * next later_c_device_status on the stream then returns LATER_ERR_TIMEOUT, and
 * the context stays usable: the same path every kernel of the library takes
 * when one of its waits runs out.
 */
later_status_t later_c_wait_selftest(later_stream_t stream, long long timeout_cycles);

/* ------------------------------------------------------------------ QR */

/* Minimum `work` (floats) and `hwork` (16-bit elements) for later_c_rgsqrf. */
later_status_t later_c_rgsqrf_bufsize(int m, int n, const later_options_t* opt, int64_t* lwork,
                                      int64_t* lhwork);

/*
 * Recursive Gram-Schmidt QR, A = Q R.
 * Replaces LATER include/LATER.h:39 later_rgsqrf (QR/later_rgsqrf.cu:62-79).
 * A (m x n, lda >= m) is overwritten by Q; R (n x n, ldr >= n) receives the
 * upper-triangular factor with a positive diagonal and zeros below it.
 * Requires m >= n >= 1 and n a multiple of 32.
 */
later_status_t later_c_rgsqrf(later_stream_t stream, int m, int n, float* A, int lda, float* R, int ldr,
                              float* work, int64_t lwork, void* hwork, int64_t lhwork,
                              const later_options_t* opt);

/*
 * later_c_rgsqrf with the matrix in host memory (no counterpart in the
 * reference, whose callers copy A to the device themselves). hA (m x n,
 * ldha) is copied to the device buffer A (lda) in chunks of columns on a
 * copy stream, each chunk converted to 16 bits there; the factorisation
 * waits for a chunk only where it first reads it. Q's columns and R's
 * columns (rows on and above the diagonal) are copied back to hQ and hR in
 * chunks as soon as the leaf that finishes them has run, while the rest of
 * the factorisation proceeds. hQ may be hA. R (device, n x n, ldr) as in
 * later_c_rgsqrf; entries of hR below the diagonal are not written. Host
 * buffers must be pinned (cudaHostAlloc / cudaHostRegister) for the copies
 * to overlap. The work is complete when `stream` reaches the point after
 * this call. The copy streams are created on the first call from a host
 * thread on a device and kept until exit.
 */
later_status_t later_c_rgsqrf_host(later_stream_t stream, int m, int n, const float* hA, int ldha, float* hQ,
                                   int ldhq, float* hR, int ldhr, float* A, int lda, float* R, int ldr, float* work,
                                   int64_t lwork, void* hwork, int64_t lhwork, const later_options_t* opt);

/* Device bytes later_c_oc_rgsqrf needs for in-core panels of `panel` columns. */
later_status_t later_c_oc_rgsqrf_bufsize(int m, int panel, const later_options_t* opt, int64_t* dev_bytes);

/*
 * Out-of-core recursive Gram-Schmidt QR: A (m x n, ldha) stays in host memory
 * and is overwritten by Q; R (n x n, ldhr) is written to host memory in full
 * (zeros below the diagonal). Replaces LATER include/LATER.h:49-51
 * later_oc_qr_rec / later_oc_qr_blk (QR/later_oc_qr.cu:29-121, with the
 * tiled host-device GEMM of BLAS/later_gemm.cu:52-189), whose signatures pass
 * the reference's Mem_pool class. The work runs through the caller's device
 * region `dev` (dev_bytes, 256-byte aligned): panels of `panel` columns (a
 * multiple of 32; 0 = the widest power-of-two multiple of 128 that fits) are
 * factored in core by rgsqrf after the projections against all earlier
 * panels' Q, which are streamed back in on a copy stream and double-buffered
 * against the tensor-core products. Host buffers must be pinned for the
 * copies to overlap. Precision and CGS2 as later_c_rgsqrf.
 */
later_status_t later_c_oc_rgsqrf(later_stream_t stream, int m, int n, float* hA, int ldha, float* hR, int ldhr,
                                 int panel, void* dev, int64_t dev_bytes, const later_options_t* opt);

/* Minimum `work` (floats) and `hwork` (16-bit elements) for later_c_rhouqr. */
later_status_t later_c_rhouqr_bufsize(int m, int n, const later_options_t* opt, int64_t* lwork,
                                      int64_t* lhwork);

/*
 * Recursive Householder QR in compact-WY form: Q = I - W Y^T, A = Q R.
 * Replaces LATER include/LATER.h:41 later_rhouqr (QR/later_rhouqr.cu:27-201).
 * A (m x n) is overwritten by Y (unit lower trapezoidal Householder vectors,
 * LAPACK dgeqrf's V); W (m x n) receives W = Y T; R (n x n) the upper factor
 * with LAPACK's sign convention and zeros below the diagonal.
 * Requires m >= n and n a multiple of 32. (The reference's 32x32 `U` scratch
 * argument is not needed: the reconstruction scratch lives in `work`.)
 */
later_status_t later_c_rhouqr(later_stream_t stream, int m, int n, float* A, int lda, float* W, int ldw,
                              float* R, int ldr, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                              const later_options_t* opt);

/* Minimum `work` (floats) and `hwork` (16-bit elements) for later_c_bhouqr. */
later_status_t later_c_bhouqr_bufsize(int m, int n, const later_options_t* opt, int64_t* lwork,
                                      int64_t* lhwork);

/*
 * Blocked Householder QR with 128-column rhouqr panels.
 * Replaces LATER include/LATER.h:45 later_bhouqr (QR/later_bhouqr.cu:88-189).
 * Outputs as later_c_rhouqr: Y (unit lower trapezoidal) in A, W (m x n,
 * ldw) with Q = I - W Y^T, R (n x n, zeros below the diagonal). The trailing
 * updates and the W merges run on the tensor cores in opt->precision (FP16,
 * BF16 or SPLIT3; the reference's FP32 SGEMMs correspond to SPLIT3); the
 * 128-column panels run in FP32 as the reference's do. W's rows above each
 * panel are zeroed before its merge. Requires m >= n and n a multiple of 32.
 * later_c_ormqr forms Q from the result (the reference's later_ormqr2).
 */
later_status_t later_c_bhouqr(later_stream_t stream, int m, int n, float* A, int lda, float* W, int ldw,
                              float* R, int ldr, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                              const later_options_t* opt);

/* Minimum `work` (floats) and `hwork` (16-bit elements) for later_c_qdwh_polar. */
later_status_t later_c_qdwh_bufsize(int m, int n, const later_options_t* opt, int64_t* lwork, int64_t* lhwork);

/*
 * Polar decomposition A = U H by the QR-based dynamically weighted Halley
 * iteration (QDWH). Replaces LATER include/LATER.h:70 later_qdwh_polar
 * (EVD/later_qdwh_polar.cu:24-110), which runs later_rgsqrf on the
 * (m + n) x n stack [sqrt(c) X; I] and one tensor-core product per step.
 * A (m x n, m >= n, n a multiple of 32) is read only; U (m x n, ldu) receives
 * the polar factor with orthonormal columns, H (n x n, ldh; may be NULL) the
 * symmetric positive semidefinite factor. The stack's QR runs with CGS2 and
 * opt->precision (FP16 / BF16 / SPLIT3; SPLIT2 is taken as SPLIT3): Q must be
 * orthonormal to working accuracy although the stack's condition number is
 * about sqrt(c), so SPLIT3 is needed for an FP32-level U. l0 > 0 is a lower
 * bound on the smallest singular value of A / ||A||_F (0: estimated as
 * 1 / ||R0^{-1}||_F from a QR of it); `symmetric` symmetrises every iterate
 * (square symmetric A only, as the reference does); tol (0: 1e-6) sets the
 * stopping test 1 - l < 5 tol, ||X_k+1 - X_k||_F < (5 tol)^(1/3); max_iter (0:
 * 10). *iterations (may be NULL) receives the number of steps taken. Host
 * code reads two norms per step, so the call synchronises the stream.
 */
later_status_t later_c_qdwh_polar(later_stream_t stream, int m, int n, const float* A, int lda, float* U, int ldu,
                                  float* H, int ldh, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                                  const later_options_t* opt, double l0, int symmetric, double tol, int max_iter,
                                  int* iterations);

/* Minimum `work` (floats) and `hwork` (16-bit elements) for later_c_sy2sb. */
later_status_t later_c_sy2sb_bufsize(int n, int nb, const later_options_t* opt, int64_t* lwork, int64_t* lhwork);

/*
 * Symmetric to band reduction B = Q^T A Q with bandwidth nb (32, 64, 96 or
 * 128; n a multiple of nb). Replaces LATER include/LATER.h:72-74
 * later_sy2sb_rec / ssytrd_sy2sb (EVD/later_sy2sb_rec.cu,
 * EVD/later_sy2sb_blocked.cu:23-186): rhouqr panels and the two-sided ZY
 * update A22 -= Y Z^T + Z Y^T, Z = A22 W - Y (W^T A22 W) / 2, on the tensor
 * cores in opt->precision (FP16 / BF16 / SPLIT3). A (n x n, both triangles
 * stored) is overwritten by B in the same full storage, zeros outside the
 * band. Y and W (n x n each, may be NULL) receive the reflectors of block
 * column i in rows i+nb.. of columns i..i+nb-1 (zeros elsewhere), so that
 * Q = prod_i (I - W_i Y_i^T).
 */
later_status_t later_c_sy2sb(later_stream_t stream, int n, int nb, float* A, int lda, float* Y, int ldy, float* W,
                             int ldw, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                             const later_options_t* opt);

/*
 * Explicit Q = I - W Y^T (first n columns), written over W, in FP32.
 * Replaces LATER include/LATER.h:43 later_ormqr and :47 later_ormqr2
 * (QR/later_ormqr.cu:18-86). `work` holds m*n floats. Unlike the reference's
 * later_ormqr, W is used as rhouqr returns it (already merged): the
 * reference repeats the top-level W merge (QR/later_ormqr.cu:27-45) that its
 * rhouqr already performed (QR/later_rhouqr.cu:150-199, the `n < ori_n`
 * guard is commented out), which would apply Q1 twice.
 */
later_status_t later_c_ormqr(later_stream_t stream, int m, int n, float* W, int ldw, const float* Y, int ldy,
                             float* work, int64_t lwork);

/* ------------------------------------------------- BLAS-3 and Cholesky */

/*
 * Workspace of the BLAS-3 / Cholesky routines: `hwork` (16-bit elements) is
 * required; `work` (floats) is optional and lets the tensor-core GEMMs split
 * K over idle SMs. `op` is 's' (rsyrk: m = n, n = k), 't' (rtrsm, leri in
 * `side`), 'm' (rtrmm) or 'p' (rpotrf: m = n).
 */
later_status_t later_c_blas3_bufsize(char op, char side, int m, int n, const later_options_t* opt, int64_t* lwork,
                                     int64_t* lhwork);

/*
 * C <- alpha A A^T + beta C on the lower triangle (C n x n, A n x k).
 * Replaces LATER include/LATER.h:62 later_rsyrk (BLAS/later_rsyrk.cu:12-93).
 * The strictly upper triangle of C is not referenced.
 */
later_status_t later_c_rsyrk(later_stream_t stream, int n, int k, float alpha, const float* A, int lda, float beta,
                             float* C, int ldc, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                             const later_options_t* opt);

/*
 * Triangular solve with a lower-triangular A, in place in B:
 *   ('l','l','n'): A X = B, A m x m;   ('l','r','t'): X A^T = B, A n x n.
 * Replaces LATER include/LATER.h:60 later_rtrsm (BLAS/later_rtrsm.cu:165-187).
 * Other flag combinations return LATER_ERR_NOT_SUPPORTED (the reference
 * silently did nothing).
 */
later_status_t later_c_rtrsm(later_stream_t stream, char uplo, char leri, char trans, int m, int n, const float* A,
                             int lda, float* B, int ldb, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                             const later_options_t* opt);

/*
 * C = A B with A m x m lower triangular, B and C m x n.
 * Replaces LATER include/LATER.h:64 later_rtrmm (BLAS/later_rtrmm.cu:14-86);
 * the reference's tempC scratch is not needed (the off-diagonal product is
 * accumulated into C by the GEMM epilogue).
 */
later_status_t later_c_rtrmm(later_stream_t stream, int m, int n, const float* A, int lda, const float* B, int ldb,
                             float* C, int ldc, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                             const later_options_t* opt);

/*
 * Lower Cholesky factor in place: A = L L^T (uplo 'l' only), any lda >= n.
 * Replaces LATER include/LATER.h:80 later_rpotrf (Cholesky/later_rpotrf.cu:68-91).
 * A non-positive pivot is reported by later_c_device_status as
 * LATER_ERR_NUMERIC. The strictly upper triangle of A is not referenced.
 */
later_status_t later_c_rpotrf(later_stream_t stream, char uplo, int n, float* A, int lda, float* work,
                              int64_t lwork, void* hwork, int64_t lhwork, const later_options_t* opt);

/* ----------------------------------------------- mixed-precision solvers */
/* No counterpart in the reference (LATER has the factorisations only). Both
 * solvers synchronise `stream` (host convergence test between iterations);
 * nrhs <= 16; X is FP64 (n x nrhs, ldx). FP64 arithmetic runs only in the
 * residual r = B - A X, A^T r and the update of X. */

typedef struct {
  int iterations;          /* refinement steps taken */
  int factor_precision;    /* later_precision_t the factorisation finally used */
  double backward_error;   /* final normwise backward error, computed in FP64 */
} later_solve_info_t;

later_status_t later_c_spd_solve_bufsize(int n, int nrhs, const later_options_t* opt, int64_t* lwork,
                                         int64_t* lhwork);

/*
 * SPD solve A X = B: rpotrf (opt->precision; a non-SPD 16-bit factorisation
 * is redone in SPLIT3), FP32 triangular solves, then FP64 iterative
 * refinement until max_c ||r_c||inf / (||A||inf ||x_c||inf + ||b_c||inf) <= tol
 * or max_iter steps. A (n x n FP32) and B are not modified.
 */
later_status_t later_c_spd_solve(later_stream_t stream, int n, int nrhs, const float* A, int lda, const float* B,
                                 int ldb, double* X, int ldx, float* work, int64_t lwork, void* hwork,
                                 int64_t lhwork, const later_options_t* opt, int max_iter, double tol,
                                 later_solve_info_t* info);

later_status_t later_c_ls_solve_bufsize(int m, int n, int nrhs, const later_options_t* opt, int64_t* lwork,
                                        int64_t* lhwork);

/*
 * Least squares min ||A X - B|| (m >= n, n a multiple of 32): rgsqrf
 * (opt->precision; SPLIT3 recommended for kappa > 1e3), X = R^-1 Q^T B, then
 * X += R^-1 Q^T (B - A X) with FP64 residuals until the backward error of the
 * augmented system, max_c ||A^T r_c||inf / (||A_aug||inf max(||r_c||inf, ||x_c||inf)
 * + ||b_c||inf), is <= tol or max_iter steps. A and B are not modified.
 */
later_status_t later_c_ls_solve(later_stream_t stream, int m, int n, int nrhs, const float* A, int lda,
                                const float* B, int ldb, double* X, int ldx, float* work, int64_t lwork,
                                void* hwork, int64_t lhwork, const later_options_t* opt, int max_iter, double tol,
                                later_solve_info_t* info);

/* ------------------------------------------------ least-squares serving */
/* No counterpart in the reference. A server owns one device, `slots` worker
 * threads with one CUDA stream each, and an HBM budget (one allocation made at
 * creation, carved per request by a first-fit pool). Requests (host A, B; the
 * FP64 solution X is written back to host memory) queue FIFO; a free worker
 * admits the head request as soon as the pool holds everything it needs, so
 * requests arriving while others run are admitted as slots and memory free
 * up and their kernels overlap on the device. Each request runs
 * later_c_ls_solve's algorithm (QR factors stay in HBM for the whole solve). */

typedef struct later_server later_server_t;

typedef struct {
  int m, n, nrhs, reserved; /* m >= n >= 32, nrhs <= 16 */
  const float* A;           /* host, column-major m x n */
  const float* B;           /* host, m x nrhs */
  double* X;                /* host, n x nrhs, receives the solution */
  int lda, ldb, ldx, reserved2;
} later_ls_request_t;

typedef struct {
  int status;               /* later_status_t of the solve */
  int iterations;
  int slot;                 /* worker that served it */
  int reserved;
  double backward_error;
  double submit_ms;         /* submit time since server creation */
  double queue_ms;          /* submit -> admitted */
  double service_ms;        /* admitted -> done */
  double latency_ms;        /* submit -> done */
} later_ls_result_t;

/* Returns NULL on failure (bad arguments or the budget allocation failed). */
later_server_t* later_c_ls_server_create(int device, int slots, int64_t hbm_budget_bytes,
                                         const later_options_t* opt, int max_iter, double tol);
/* Queues a request; returns a ticket >= 0, or -later_status_t (a request
 * larger than the whole budget is refused with -LATER_ERR_WORKSPACE). The
 * host buffers must stay valid until later_c_ls_server_wait returns. They may
 * be pageable (the driver stages each copy); pinned buffers (cudaHostAlloc /
 * cudaHostRegister) let a slot's copies run asynchronously with the device. */
int64_t later_c_ls_server_submit(later_server_t* s, const later_ls_request_t* req);
/* Blocks until the request is done and fills `out`. */
later_status_t later_c_ls_server_wait(later_server_t* s, int64_t ticket, later_ls_result_t* out);
/* Bytes of the HBM budget currently held by admitted requests. */
int64_t later_c_ls_server_hbm_in_use(later_server_t* s);
/* Largest number of budget bytes held at once since the server was created. */
int64_t later_c_ls_server_hbm_peak(later_server_t* s);
/* Drains the queue, joins the workers and frees the budget. */
void later_c_ls_server_destroy(later_server_t* s);

/* ---------------------------------------------------------- batched QR */
/* No counterpart in the reference. Many independent FP32 matrices of uneven
 * sizes (m >= n, n <= 256) factored A_i = Q_i R_i in one persistent-kernel
 * launch: Q_i overwrites A_i, R_i (n x n) gets the upper factor with a
 * positive diagonal and zeros below it. */

typedef struct {
  float* A;     /* device, column-major m x n */
  float* R;     /* device, n x n */
  int64_t lda;
  int64_t ldr;
  int m;
  int n;
} later_qr_item_t;

/* Device bytes of the plan for `count` matrices. */
int64_t later_c_batched_plan_bytes(int count);

/* Sorts the matrices by decreasing cost (2 n^2 m) and uploads their
 * descriptors into `plan` (device). Synchronises `stream`. */
later_status_t later_c_batched_qr_plan(later_stream_t stream, int count, const later_qr_item_t* items, void* plan,
                                       int64_t plan_bytes);

/* Factors every matrix of the plan: one counter reset (`queue`, one device
 * int) and one launch, so it can be captured in a CUDA graph. `status`
 * (device, count ints, may be NULL) receives 0 or LATER_ERR_NUMERIC per
 * matrix (a 32-column panel whose Cholesky QR broke down: kappa too large
 * for CholQR2 in FP32). `variant` picks the tile shape (0 .. 3, see
 * later_gb300.autotune); -1 uses variant 0. */
later_status_t later_c_batched_qr_run(later_stream_t stream, int count, const void* plan, int* queue, int* status,
                                      int variant);

/* --------------------------------------------------------- building blocks */

/*
 * Tensor-core GEMM on 16-bit operands with FP32 accumulation:
 *   D = alpha * op(A) * op(B) + beta * C      (op(X) = X or X^T by 'N' / 'T')
 * A, B hold FP16 (precision FP16) or BF16 (precision BF16) elements; lda, ldb
 * must be multiples of 8 and the pointers 16-byte aligned. C and D are FP32
 * and may alias. `work` (floats) holds split-K partial sums; lwork = 0 turns
 * split-K off. This is the kernel under every trailing update of
 * QR/later_rgsqrf.cu:45-56 (cublasGemmEx sites in the reference).
 */
later_status_t later_c_gemm16(later_stream_t stream, char transa, char transb, int m, int n, int k,
                              float alpha, const void* A, int lda, const void* B, int ldb, float beta,
                              const float* C, int ldc, float* D, int ldd, int precision, float* work,
                              int64_t lwork);

/*
 * later_c_gemm16 without a caller workspace (no counterpart in the reference).
 * For callers that cannot allocate device memory (a host framework whose own
 * pool owns all device memory and forbids plug-ins from calling the
 * allocator, or a latency-critical path that cannot afford cudaMalloc's
 * implicit synchronisation): the split-K scratch is a fixed device array of
 * LATER_NOALLOC_SCRATCH_FLOATS floats (16 MiB) inside this library, held by
 * every GPU that loads it until exit. The call allocates nothing. The first
 * call on a device looks up the array's address; make it before any stream
 * capture. Any output size is accepted: K is split only as far as the array
 * holds the partial tiles (not at all when they do not fit). All calls share
 * the array: calls whose kernels overlap on the GPU race on it.
 */
#define LATER_NOALLOC_SCRATCH_FLOATS 4194304
later_status_t later_c_gemm16_noalloc(later_stream_t stream, char transa, char transb, int m, int n, int k,
                                      float alpha, const void* A, int lda, const void* B, int ldb, float beta,
                                      const float* C, int ldc, float* D, int ldd, int precision);

/*
 * FP32 -> 16-bit conversion of an m x n column-major block (the role of
 * util/util.cu:24-32 s2h). precision FP16 / BF16 writes `hi`; SPLIT3 writes
 * hi = fp16(x) and lo = fp16((x - hi) * 2048).
 */
later_status_t later_c_convert(later_stream_t stream, int m, int n, const float* A, int lda, void* hi,
                               void* lo, int ldh, int precision);

/* ------------------------------------------------------------ tracing */

/* Cumulative number of kernels this library has launched (all streams). */
uint64_t later_c_launch_count(void);

typedef struct {
  double gemm_flops;      /* algorithmic flops (2 m n k) of the tensor-core GEMMs */
  double gemm_ms;         /* their summed device time */
  int64_t gemm_launches;
  double top_gemm_flops;  /* the largest single GEMM launch ... */
  double top_gemm_ms;     /* ... and its device time */
  double panel_ms;        /* FP32 TSQR panels (reduction tree + apply) */
  int64_t panel_launches;
  double leaf_gemm_flops; /* FP32 leaf projections */
  double leaf_gemm_ms;
  int64_t leaf_gemm_launches;
  double other_ms;        /* conversions, fills, small solves */
  int64_t other_launches;
} later_trace_t;

/* Starts event tracing of every launch group on its stream (clears old records). */
void later_c_trace_begin(void);
/* Stops tracing, waits for the recorded events and returns the per-class sums. */
later_status_t later_c_trace_end(later_trace_t* out);

#ifdef __cplusplus
}
#endif

#endif /* LATER_C_H */

// The reference LATER on the GPU, for parity checks and as the same-GPU
// comparator. Test and benchmark infrastructure only: nothing in the product
// library links or loads this file's output.
//
// The reference's own device kernels (mgs_kernel2 from QR/panel.cu, s2h from
// util/util.cu) are compiled unchanged from its sources into cubins by
// oracle/build_ref.py and loaded here through the driver API. Its host code
// is restated below, call for call, with the same cuBLAS / cuSOLVER calls it
// makes (GemmEx FP16 -> FP32 with CUBLAS_GEMM_DEFAULT_TENSOR_OP, Sgemm,
// SgemmStridedBatched with the output aliasing the input, Strsm, Spotrf), so
// the arithmetic is the reference's: its FP32 SIMT panels and the vendor
// library's tensor-core GEMMs on this GPU. The cuSOLVER calls the reference's
// QR test uses as its FP32 comparator (test/test_qr.cu:184-206) are exported
// as well.
//
// Restated host code, with the reference lines it follows:
//   ref_rgsqrf                QR/later_rgsqrf.cu:25-79   (qr, later_rgsqrf)
//   mgs_caqr_panel_256x128    QR/panel.cu:10-63
//   mgs_caqr_panel_256x32     QR/panel.cu:65-134
//   ref_rpotrf                Cholesky/later_rpotrf.cu:22-91 (l_potrf; timers and prints dropped)
//   trsm_l_r_t                BLAS/later_rtrsm.cu:126-163
//   syrk                      BLAS/later_rsyrk.cu:12-77
#include <cublas_v2.h>
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cstdint>
#include <cstdio>
#include <string>

namespace {

struct Ref {
  bool ready = false;
  CUmodule panel = nullptr, util = nullptr;
  CUfunction mgs_kernel2 = nullptr, s2h = nullptr;
  cublasHandle_t cb = nullptr;
  cusolverDnHandle_t cs = nullptr;
  cudaStream_t st = nullptr;
  int* dev_info = nullptr;
  float* potrf_work = nullptr;  // LWORK floats, the reference's fixed Spotrf workspace
  int err = 0;                  // first failure: 1 CUDA, 2 cuBLAS, 3 cuSOLVER, 4 driver
};
Ref g;

constexpr int kPotrfLwork = 65536;  // Cholesky/later_rpotrf.cu:8
constexpr int kPotrfBlock = 2048;   // Cholesky/later_rpotrf.cu:7
constexpr int kSyrkBlock = 2048;    // BLAS/later_rsyrk.cu:5
constexpr int kTrsmBlock = 256;     // BLAS/later_rtrsm.cu:5

void fail(int code) {
  if (!g.err) g.err = code;
}
void ck(cudaError_t e) {
  if (e != cudaSuccess) fail(1);
}
void ck(cublasStatus_t e) {
  if (e != CUBLAS_STATUS_SUCCESS) fail(2);
}
void ck(cusolverStatus_t e) {
  if (e != CUSOLVER_STATUS_SUCCESS) fail(3);
}
void ck(CUresult e) {
  if (e != CUDA_SUCCESS) fail(4);
}

void launch(CUfunction f, dim3 grid, dim3 block, void** args) {
  ck(cuLaunchKernel(f, grid.x, grid.y, grid.z, block.x, block.y, block.z, 0, reinterpret_cast<CUstream>(g.st), args,
                    nullptr));
}

void s2h(dim3 grid, int m, int n, const float* as, int ldas, __half* ah, int ldah) {
  void* args[] = {&m, &n, &as, &ldas, &ah, &ldah};
  launch(g.s2h, grid, dim3(32, 32), args);
}

void mgs_kernel2(int blocks, int m, int n, float* A, int lda, float* R, int ldr) {
  void* args[] = {&m, &n, &A, &lda, &R, &ldr};
  launch(g.mgs_kernel2, dim3(blocks), dim3(32, 32), args);
}

const float sone = 1.0f, szero = 0.0f, snegone = -1.0f;

// QR/panel.cu:65-134
void mgs_caqr_panel_256x32(int m, int n, float* A, int lda, float* R, int ldr, float* work) {
  if (n != 32) {
    fail(5);
    return;
  }
  if (m <= 256) {
    mgs_kernel2(1, m, n, A, lda, R, ldr);
    return;
  }
  if (m % 256 == 0) {
    const int ldwork = m / 256 * 32, mm = m / 256 * 32;
    mgs_kernel2(m / 256, m, n, A, lda, work, ldwork);
    mgs_caqr_panel_256x32(mm, n, work, ldwork, R, ldr, work + static_cast<int64_t>(ldwork) * n);
    ck(cublasSgemmStridedBatched(g.cb, CUBLAS_OP_N, CUBLAS_OP_N, 256, 32, 32, &sone, A, lda, 256, work, ldwork, 32,
                                 &szero, A, lda, 256, m / 256));
  } else {
    const int nb = m / 256, r = m % 256;
    const int ldwork = m / 256 * 32 + 32, mm = m / 256 * 32 + 32;
    mgs_kernel2(m / 256 + 1, m, n, A, lda, work, ldwork);
    mgs_caqr_panel_256x32(mm, n, work, ldwork, R, ldr, work + static_cast<int64_t>(ldwork) * n);
    ck(cublasSgemmStridedBatched(g.cb, CUBLAS_OP_N, CUBLAS_OP_N, 256, 32, 32, &sone, A, lda, 256, work, ldwork, 32,
                                 &szero, A, lda, 256, nb));
    ck(cublasSgemm(g.cb, CUBLAS_OP_N, CUBLAS_OP_N, r, 32, 32, &sone, A + nb * 256, lda, work + nb * 32, ldwork,
                   &szero, A + nb * 256, lda));
  }
}

// QR/panel.cu:10-63
void mgs_caqr_panel_256x128(int m, int n, float* A, int lda, float* R, int ldr, float* work) {
  if (m < 256 || n != 128) {
    fail(5);
    return;
  }
  mgs_caqr_panel_256x32(m, 32, A, lda, R, ldr, work);
  ck(cublasSgemm(g.cb, CUBLAS_OP_T, CUBLAS_OP_N, 32, 32, m, &sone, A, lda, A + 32 * lda, lda, &szero, R + 32 * ldr,
                 ldr));
  ck(cublasSgemm(g.cb, CUBLAS_OP_N, CUBLAS_OP_N, m, 32, 32, &snegone, A, lda, R + 32 * ldr, ldr, &sone, A + 32 * lda,
                 lda));
  mgs_caqr_panel_256x32(m, 32, A + 32 * lda, lda, R + 32 + 32 * ldr, ldr, work);
  ck(cublasSgemm(g.cb, CUBLAS_OP_T, CUBLAS_OP_N, 64, 64, m, &sone, A, lda, A + 64 * lda, lda, &szero, R + 64 * ldr,
                 ldr));
  ck(cublasSgemm(g.cb, CUBLAS_OP_N, CUBLAS_OP_N, m, 64, 64, &snegone, A, lda, R + 64 * ldr, ldr, &sone, A + 64 * lda,
                 lda));
  A = A + 64 * lda;
  R = R + 64 * ldr + 64;
  mgs_caqr_panel_256x32(m, 32, A, lda, R, ldr, work);
  ck(cublasSgemm(g.cb, CUBLAS_OP_T, CUBLAS_OP_N, 32, 32, m, &sone, A, lda, A + 32 * lda, lda, &szero, R + 32 * ldr,
                 ldr));
  ck(cublasSgemm(g.cb, CUBLAS_OP_N, CUBLAS_OP_N, m, 32, 32, &snegone, A, lda, R + 32 * ldr, ldr, &sone, A + 32 * lda,
                 lda));
  mgs_caqr_panel_256x32(m, 32, A + 32 * lda, lda, R + 32 + 32 * ldr, ldr, work);
}

// QR/later_rgsqrf.cu:25-60 (NMIN 128)
void qr(int m, int n, float* A, int lda, float* R, int ldr, float* work, __half* hwork) {
  if (n <= 128) {
    mgs_caqr_panel_256x128(m, n, A, lda, R, ldr, work);
    return;
  }
  qr(m, n / 2, A, lda, R, ldr, work, hwork);
  __half* Ah = hwork;
  __half* Bh = hwork + static_cast<int64_t>(m) * (n / 2);
  const dim3 grid((m + 31) / 32, (n + 31) / 32);
  s2h(grid, m, n / 2, A, m, Ah, m);
  s2h(grid, m, n / 2, A + static_cast<int64_t>(n / 2) * lda, m, Bh, m);
  ck(cublasGemmEx(g.cb, CUBLAS_OP_T, CUBLAS_OP_N, n / 2, n / 2, m, &sone, Ah, CUDA_R_16F, lda, Bh, CUDA_R_16F, lda,
                  &szero, R + static_cast<int64_t>(n / 2) * ldr, CUDA_R_32F, ldr, CUBLAS_COMPUTE_32F,
                  CUBLAS_GEMM_DEFAULT_TENSOR_OP));
  const dim3 grid2((n + 31) / 32, (n + 31) / 31);  // as launched at :50
  s2h(grid2, n / 2, n / 2, R + static_cast<int64_t>(n / 2) * ldr, ldr, Bh, n / 2);
  ck(cublasGemmEx(g.cb, CUBLAS_OP_N, CUBLAS_OP_N, m, n / 2, n / 2, &snegone, Ah, CUDA_R_16F, m, Bh, CUDA_R_16F,
                  n / 2, &sone, A + static_cast<int64_t>(n / 2) * lda, CUDA_R_32F, lda, CUBLAS_COMPUTE_32F,
                  CUBLAS_GEMM_DEFAULT_TENSOR_OP));
  qr(m, n / 2, A + static_cast<int64_t>(n / 2) * lda, lda, R + n / 2 + static_cast<int64_t>(n / 2) * ldr, ldr, work,
     hwork);
}

// BLAS/later_rtrsm.cu:126-163 (X L^T = B)
void trsm_l_r_t(int m, int n, float* A, int lda, float* B, int ldb, __half* hwork) {
  if (n <= kTrsmBlock) {
    ck(cublasStrsm(g.cb, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, m, n, &sone, A,
                   lda, B, ldb));
    return;
  }
  trsm_l_r_t(m, n / 2, A, lda, B, ldb, hwork);
  __half* Ah = hwork;
  __half* Bh = hwork + static_cast<int64_t>(n / 2) * (n / 2);
  s2h(dim3((n / 2 + 31) / 32, (n / 2 + 31) / 32), n / 2, n / 2, A + n / 2, lda, Ah, n / 2);
  s2h(dim3((m + 31) / 32, (n / 2 + 31) / 32), m, n / 2, B, ldb, Bh, m);
  ck(cublasGemmEx(g.cb, CUBLAS_OP_N, CUBLAS_OP_T, m, n / 2, n / 2, &snegone, Bh, CUDA_R_16F, m, Ah, CUDA_R_16F, n / 2,
                  &sone, B + static_cast<int64_t>(n / 2) * ldb, CUDA_R_32F, ldb, CUBLAS_COMPUTE_32F,
                  CUBLAS_GEMM_DEFAULT_TENSOR_OP));
  trsm_l_r_t(m, n / 2, A + static_cast<int64_t>(n / 2) * lda + n / 2, lda, B + static_cast<int64_t>(n / 2) * ldb, ldb,
             hwork);
}

// BLAS/later_rsyrk.cu:12-77 (C <- alpha A A^T + beta C; the leaf writes the full square block)
void syrk(int n, int k, float alpha, float* A, int lda, float beta, float* C, int ldc, __half* hwork) {
  if (n <= kSyrkBlock) {
    __half* ah = hwork;
    s2h(dim3((n + 1) / 32, (k + 1) / 32), n, k, A, lda, ah, n);
    ck(cublasGemmEx(g.cb, CUBLAS_OP_N, CUBLAS_OP_T, n, n, k, &alpha, ah, CUDA_R_16F, n, ah, CUDA_R_16F, n, &beta, C,
                    CUDA_R_32F, ldc, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT_TENSOR_OP));
    return;
  }
  syrk(n / 2, k, alpha, A, lda, beta, C, ldc, hwork);
  __half* Ah = hwork;
  __half* Bh = hwork + static_cast<int64_t>(n / 2) * k;
  const dim3 grid((n / 2 + 1) / 32, (k + 1) / 32);
  s2h(grid, n / 2, k, A + n / 2, lda, Ah, n / 2);
  s2h(grid, n / 2, k, A, lda, Bh, n / 2);
  ck(cublasGemmEx(g.cb, CUBLAS_OP_N, CUBLAS_OP_T, n / 2, n / 2, k, &alpha, Ah, CUDA_R_16F, n / 2, Bh, CUDA_R_16F,
                  n / 2, &beta, C + n / 2, CUDA_R_32F, ldc, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT_TENSOR_OP));
  syrk(n / 2, k, alpha, A + n / 2, lda, beta, C + n / 2 + static_cast<int64_t>(ldc / 2) * n, ldc, hwork);
}

// Cholesky/later_rpotrf.cu:22-66 (the recursion passes n as the leading dimension: lda == n)
void l_potrf(int n, float* A, int lda, __half* hwork) {
  if (n <= kPotrfBlock) {
    ck(cusolverDnSpotrf(g.cs, CUBLAS_FILL_MODE_LOWER, n, A, lda, g.potrf_work, kPotrfLwork, g.dev_info));
    return;
  }
  l_potrf(n / 2, A, n, hwork);
  trsm_l_r_t(n / 2, n / 2, A, n, A + n / 2, n, hwork);
  syrk(n / 2, n / 2, -1.0f, A + n / 2, n, 1.0f, A + static_cast<int64_t>(n / 2) * n + n / 2, n, hwork);
  l_potrf(n / 2, A + static_cast<int64_t>(n / 2) * n + n / 2, n, hwork);
}

}  // namespace

extern "C" {

// Loads the reference's kernels from `dir` (panel.cubin, util.cubin) into the
// current device's primary context and binds cuBLAS / cuSOLVER to `stream`.
// Returns 0 on success.
int ref_init(const char* dir, void* stream) {
  if (g.ready) {
    g.st = static_cast<cudaStream_t>(stream);
    cublasSetStream(g.cb, g.st);
    cusolverDnSetStream(g.cs, g.st);
    return 0;
  }
  g.err = 0;
  ck(cudaFree(nullptr));  // the runtime's primary context becomes current
  const std::string d(dir);
  ck(cuModuleLoad(&g.panel, (d + "/panel.cubin").c_str()));
  ck(cuModuleLoad(&g.util, (d + "/util.cubin").c_str()));
  if (g.err) return g.err;
  ck(cuModuleGetFunction(&g.mgs_kernel2, g.panel, "_Z11mgs_kernel2iiPfiS_i"));
  ck(cuModuleGetFunction(&g.s2h, g.util, "_Z3s2hiiPfiP6__halfi"));
  ck(cublasCreate(&g.cb));
  ck(cusolverDnCreate(&g.cs));
  ck(cudaMalloc(&g.dev_info, sizeof(int)));
  ck(cudaMalloc(&g.potrf_work, sizeof(float) * kPotrfLwork));
  if (g.err) return g.err;
  g.st = static_cast<cudaStream_t>(stream);
  ck(cublasSetStream(g.cb, g.st));
  ck(cusolverDnSetStream(g.cs, g.st));
  g.ready = g.err == 0;
  return g.err;
}

// later_rgsqrf (QR/later_rgsqrf.cu:62-79): like the reference, the recursion
// uses m as the leading dimension of A. Needs n = 128 * 2^k, m a multiple of
// 256, work >= m/256*32*32*2 floats, hwork >= m*n halves.
int ref_rgsqrf(int m, int n, float* A, float* R, int ldr, float* work, void* hwork) {
  if (!g.ready) return -1;
  g.err = 0;
  qr(m, n, A, m, R, ldr, work, static_cast<__half*>(hwork));
  return g.err;
}

// later_rpotrf('l', ...) (Cholesky/later_rpotrf.cu:68-91): lda must equal n;
// hwork >= n/2 * n halves (test/test_potrf.cu:74). Returns cuSOLVER's info of
// the last leaf through *info (synchronises the stream).
int ref_rpotrf(int n, float* A, void* hwork, int* info) {
  if (!g.ready) return -1;
  g.err = 0;
  ck(cudaMemsetAsync(g.dev_info, 0, sizeof(int), g.st));
  l_potrf(n, A, n, static_cast<__half*>(hwork));
  if (info) {
    ck(cudaMemcpyAsync(info, g.dev_info, sizeof(int), cudaMemcpyDeviceToHost, g.st));
    ck(cudaStreamSynchronize(g.st));
  }
  return g.err;
}

// Workspace cuSOLVER's Spotrf asks for at n (the reference passes 65536).
int ref_spotrf_bufsize(int n, float* A, int lda, int* lwork) {
  if (!g.ready) return -1;
  return cusolverDnSpotrf_bufferSize(g.cs, CUBLAS_FILL_MODE_LOWER, n, A, lda, lwork) == CUSOLVER_STATUS_SUCCESS ? 0
                                                                                                               : 3;
}

// The reference QR test's FP32 comparator (test/test_qr.cu:184-206):
// cusolverDnSgeqrf on the same matrix. Also used for the FP32 Cholesky
// comparator (cusolverDnSpotrf).
int ref_sgeqrf_bufsize(int m, int n, float* A, int lda, int* lwork) {
  if (!g.ready) return -1;
  return cusolverDnSgeqrf_bufferSize(g.cs, m, n, A, lda, lwork) == CUSOLVER_STATUS_SUCCESS ? 0 : 3;
}

int ref_sgeqrf(int m, int n, float* A, int lda, float* tau, float* work, int lwork, int* dinfo) {
  if (!g.ready) return -1;
  return cusolverDnSgeqrf(g.cs, m, n, A, lda, tau, work, lwork, dinfo) == CUSOLVER_STATUS_SUCCESS ? 0 : 3;
}

int ref_spotrf(int n, float* A, int lda, float* work, int lwork, int* dinfo) {
  if (!g.ready) return -1;
  return cusolverDnSpotrf(g.cs, CUBLAS_FILL_MODE_LOWER, n, A, lda, work, lwork, dinfo) == CUSOLVER_STATUS_SUCCESS ? 0
                                                                                                                 : 3;
}

}  // extern "C"

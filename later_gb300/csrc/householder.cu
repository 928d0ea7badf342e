// Householder reconstruction for the rhouqr leaf, and the explicit-Q former.
//
// The reference's rhouqr leaf (QR/later_rhouqr.cu:56-78, 233-276) factors a
// 32-column panel with Householder TSQR into an explicit Q, then recovers the
// compact-WY form Q = I - W Y^T from it: an LU without pivoting of I - Q
// (cusolverDnSgetrf) gives Y = L and U, then W = (I - Q) Y1^{-T} (cublasStrsm).
// Each leaf also cudaMalloc'ed its getrf scratch and never freed it (:248-249).
//
// Here the same reconstruction ("Reconstructing Householder vectors from
// Tall-Skinny QR", Ballard, Demmel, Grigori, Jacquelin, Nguyen, Solomonik,
// IPDPS 2014) runs in two allocation-free kernels, with that paper's sign
// choice: column k of Q is multiplied by s_k = -sign of the k-th pivot
// candidate, so every pivot of the LU of (I - Q S) is 1 + |.| >= 1 (the
// reference's S = I can meet a zero pivot). The result is the Householder
// form LAPACK's dgeqrf computes: R' = S R has R'_kk = -sign(.) ||.||, Y is
// unit lower trapezoidal, T = U Y1^{-T} is upper triangular and W = Y T.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "householder.cuh"
#include "runtime.cuh"

namespace later {

namespace {

constexpr int PB = 32;

__device__ __forceinline__ void put16(void* base, void* lo, int64_t o, float v, int mode) {
  if (!base) return;
  if (mode == 1) {
    reinterpret_cast<__nv_bfloat16*>(base)[o] = __float2bfloat16_rn(v);
  } else {
    const __half h = __float2half_rn(v);
    reinterpret_cast<__half*>(base)[o] = h;
    if (mode == 2) reinterpret_cast<__half*>(lo)[o] = __float2half_rn((v - __half2float(h)) * 2048.f);
  }
}

// One warp. Lane j owns column j of the top 32x32 block of Q (G_j), eliminated
// in place. Writes U (upper), s, T = U Y1^{-T} to `hr`, Y1 (unit lower) into
// the top block of A, and flips the rows of R by s.
__global__ void __launch_bounds__(32) hr_lu_kernel(int nc, float* A, int64_t lda, float* R, int64_t ldr,
                                                   HrScratch hr) {
  __shared__ float Ls[PB][PB + 1];  // L[r][k]
  __shared__ float Us[PB][PB + 1];  // U[i][j]
  __shared__ float sgn[PB];
  const int j = threadIdx.x;
  float g[PB];
#pragma unroll
  for (int r = 0; r < PB; ++r) g[r] = (j < nc && r < nc) ? A[r + static_cast<int64_t>(j) * lda] : 0.f;
#pragma unroll 1
  for (int k = 0; k < nc; ++k) {
    if (j == k) {
      float gk = 0.f;
#pragma unroll
      for (int r = 0; r < PB; ++r)
        if (r == k) gk = g[r];
      const float s = (gk >= 0.f) ? -1.f : 1.f;
      const float piv = 1.f - s * gk;  // = 1 + |gk|
      sgn[k] = s;
#pragma unroll
      for (int r = 0; r < PB; ++r) {
        if (r < k) Us[r][k] = -s * g[r];
        else if (r == k) Us[k][k] = piv;
        else {
          Ls[r][k] = (-s * g[r]) / piv;
          Us[r][k] = 0.f;
        }
      }
    }
    __syncwarp();
    if (j > k && j < nc) {
      const float gk = [&] {
        float v = 0.f;
#pragma unroll
        for (int r = 0; r < PB; ++r)
          if (r == k) v = g[r];
        return v;
      }();
#pragma unroll
      for (int r = 0; r < PB; ++r)
        if (r > k && r < nc) g[r] -= Ls[r][k] * gk;
    }
    __syncwarp();
  }
  // Y1 = unit lower L into the top block of A; S R into R; U, s to scratch.
  if (j < nc) {
#pragma unroll
    for (int r = 0; r < PB; ++r)
      if (r < nc) {
        A[r + static_cast<int64_t>(j) * lda] = (r > j) ? Ls[r][j] : (r == j ? 1.f : 0.f);
        hr.U[r + j * PB] = (r <= j) ? Us[r][j] : 0.f;
      }
    hr.s[j] = sgn[j];
  }
  __syncwarp();
  if (j < nc) {
    const float sj = sgn[j];
    for (int c = 0; c < nc; ++c) R[j + static_cast<int64_t>(c) * ldr] *= sj;  // row j of R
  }
  // T = U Y1^{-T}: lane i solves row i of T from T Y1^T = U (Y1^T unit upper).
  if (j < nc) {
    float t[PB];
#pragma unroll
    for (int c = 0; c < PB; ++c) {
      float v = (c < nc) ? ((j <= c) ? Us[j][c] : 0.f) : 0.f;
#pragma unroll
      for (int q = 0; q < PB; ++q)
        if (q < c) v -= t[q] * ((c > q) ? Ls[c][q] : 0.f);
      t[c] = v;
    }
#pragma unroll
    for (int c = 0; c < PB; ++c)
      if (c < nc) hr.T[j + c * PB] = (c >= j) ? t[c] : 0.f;
  }
}

// Row-parallel part: for rows >= nc, Y_r = -(Q_r S) U^{-1}; for every row,
// W_r = Y_r T. Writes Y into A, W into W, and their 16-bit copies.
__global__ void __launch_bounds__(256) hr_apply_kernel(int m, int nc, float* A, int64_t lda, float* W,
                                                       int64_t ldw, void* yh, void* yl, void* wh, void* wl,
                                                       int64_t ldh, int mode, HrScratch hr) {
  __shared__ float Us[PB][PB + 1];
  __shared__ float Ts[PB][PB + 1];
  __shared__ float ss[PB];
  for (int e = threadIdx.x; e < PB * PB; e += blockDim.x) {
    Us[e % PB][e / PB] = hr.U[e];
    Ts[e % PB][e / PB] = hr.T[e];
  }
  if (threadIdx.x < PB) ss[threadIdx.x] = hr.s[threadIdx.x];
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  float y[PB];
#pragma unroll
  for (int c = 0; c < PB; ++c) y[c] = (c < nc) ? A[r + static_cast<int64_t>(c) * lda] : 0.f;
  if (r >= nc) {
    // y U = -q S, U upper: forward substitution over columns.
#pragma unroll
    for (int c = 0; c < PB; ++c) {
      if (c < nc) {
        float v = -ss[c] * y[c];
#pragma unroll
        for (int q = 0; q < PB; ++q)
          if (q < c) v -= y[q] * Us[q][c];
        y[c] = v / Us[c][c];
      }
    }
  }
#pragma unroll
  for (int c = 0; c < PB; ++c) {
    if (c >= nc) break;
    float w = 0.f;
#pragma unroll
    for (int q = 0; q < PB; ++q)
      if (q <= c) w += y[q] * Ts[q][c];
    const int64_t oa = r + static_cast<int64_t>(c) * lda;
    A[oa] = y[c];
    W[r + static_cast<int64_t>(c) * ldw] = w;
    const int64_t oh = r + static_cast<int64_t>(c) * ldh;
    put16(yh, yl, oh, y[c], mode);
    put16(wh, wl, oh, w, mode);
  }
}

// Q = I - W Y1^T for the first n columns (Y1 = top n x n block of Y, unit
// lower). 64x64 output tiles, FP32, inner dimension limited to k <= column.
__global__ void __launch_bounds__(256) form_q_kernel(int m, int n, const float* __restrict__ W, int64_t ldw,
                                                     const float* __restrict__ Y, int64_t ldy, float* Q,
                                                     int64_t ldq) {
  __shared__ float Ws[64][65];
  __shared__ float Ys[64][65];
  const int r0 = blockIdx.x * 64, c0 = blockIdx.y * 64;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  const int kend = min(n, c0 + 64);
  for (int k0 = 0; k0 < kend; k0 += 64) {
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 64; e += 256) {
      const int i = e % 64, k = e / 64;
      const int kk = k0 + k;
      Ws[i][k] = (r0 + i < m && kk < n) ? W[r0 + i + static_cast<int64_t>(kk) * ldw] : 0.f;
      // Y1[c][kk]: unit lower triangular block.
      const int c = c0 + i;
      float yv = 0.f;
      if (c < n && kk < n) yv = (kk < c) ? Y[c + static_cast<int64_t>(kk) * ldy] : (kk == c ? 1.f : 0.f);
      Ys[i][k] = yv;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < 64; ++k) {
      float wr[4], yr[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        wr[u] = Ws[tx + 16 * u][k];
        yr[u] = Ys[ty + 16 * u][k];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] += wr[u] * yr[v];
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = r0 + tx + 16 * u, c = c0 + ty + 16 * v;
      if (i < m && c < n) Q[i + static_cast<int64_t>(c) * ldq] = (i == c ? 1.f : 0.f) - acc[u][v];
    }
}

}  // namespace

later_status_t householder_reconstruct(cudaStream_t st, int m, int nc, float* A, int64_t lda, float* W, int64_t ldw,
                                       float* R, int64_t ldr, void* yh, void* yl, void* wh, void* wl, int64_t ldh,
                                       int out_prec, HrScratch hr) {
  if (nc < 1 || nc > PB || m < nc) return LATER_ERR_INVALID_ARG;
  const int mode = out_prec == LATER_PREC_BF16 ? 1 : (out_prec == LATER_PREC_SPLIT3 ? 2 : 0);
  TraceScope trace(st, TRACE_PANEL);
  hr_lu_kernel<<<1, 32, 0, st>>>(nc, A, lda, R, ldr, hr);
  note_launch();
  LATER_CHECK_CUDA(cudaGetLastError());
  hr_apply_kernel<<<(m + 255) / 256, 256, 0, st>>>(m, nc, A, lda, W, ldw, yh, yl, wh, wl, ldh, mode, hr);
  note_launch();
  return cuda_status(cudaGetLastError());
}

later_status_t form_q(cudaStream_t st, int m, int n, const float* W, int64_t ldw, const float* Y, int64_t ldy,
                      float* Q, int64_t ldq) {
  if (m <= 0 || n <= 0) return LATER_OK;
  if ((n + 63) / 64 > 65535) return LATER_ERR_NOT_SUPPORTED;
  TraceScope trace(st, TRACE_LEAF_GEMM, 1.0 * m * n * n);
  form_q_kernel<<<dim3((m + 63) / 64, (n + 63) / 64), 256, 0, st>>>(m, n, W, ldw, Y, ldy, Q, ldq);
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace later

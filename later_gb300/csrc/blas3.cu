// Recursive BLAS-3 (rsyrk, rtrsm, rtrmm) and recursive Cholesky (rpotrf).
//
// Reference structure (all split the dimension in half and run the
// off-diagonal product as an FP16 cublasGemmEx on s2h copies):
//   later_rsyrk  BLAS/later_rsyrk.cu:12-93   leaf n <= 2048: full square GemmEx
//   later_rtrsm  BLAS/later_rtrsm.cu:75-187  leaf <= 256: cublasStrsm; only
//                ('l','l','n') and ('l','r','t'); other flags are a silent no-op
//   later_rtrmm  BLAS/later_rtrmm.cu:14-86   leaf <= 256: cublasStrmm; GemmEx
//                into tempC, then cublasSgeam C2 += tempC
//   later_rpotrf Cholesky/later_rpotrf.cu:22-91 leaf <= 2048: cusolverDnSpotrf,
//                off-diagonal later_rtrsm('l','r','t'), trailing later_rsyrk
// Here:
//   * rsyrk is one tensor-core NT launch over the lower tiles only (tiles above
//     the diagonal exit at once), alpha / beta in the epilogue;
//   * the leaves are FP32 kernels of this file (substitution TRSM, TRMM, and a
//     one-CTA Cholesky with a pivot check that reports LATER_ERR_NUMERIC);
//   * in rpotrf, the parts the reference runs in FP32 (updates below its
//     cuSOLVER / cublasStrsm block sizes) run as SPLIT3 tensor-core products
//     (hi + lo operands, FP32-level), and the triangular solves with at least
//     kInvMinRows rows are products with the inverse of the factor's 128-column
//     diagonal block, inverted once, all blocks of a node in one launch
//     (trtri_blocks_kernel); where such a solve splits 256 columns into two
//     128-column blocks, it is one product with the 256-column block's inverse
//     (inv256_kernel, built from the two halves' inverses); smaller solves keep
//     the FP32 substitution leaf;
//   * the blocks the reference hands to cusolverDnSpotrf (at most 2048
//     columns) are factored by a blocked right-looking loop: per 128-column
//     block the Cholesky leaf, one solve launch for all rows below, one SPLIT3
//     lower-triangle update;
//   * rtrmm adds L21 B1 into C2 in the GEMM epilogue (beta = 1): no tempC;
//   * 16-bit operand copies are written by the producing leaf (solved X) or
//     converted once per operand block right before its GEMM;
//   * leading dimensions are honoured (the reference's rpotrf assumes lda == n).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <vector>

#include "blas3.cuh"
#include "dense_dev.cuh"
#include "panel.cuh"
#include "ptx.cuh"
#include "runtime.cuh"

namespace later {

namespace {

constexpr int NB = 128;  // leaf size of the triangular solves / products / Cholesky
// Below these sizes the reference runs pure FP32 (cublasStrsm / cublasStrmm
// leaves of 256, BLAS/later_rtrsm.cu:5, BLAS/later_rtrmm.cu:5; cuSOLVER Spotrf
// leaves of 2048, Cholesky/later_rpotrf.cu:7): the recursion below them uses
// FP32 SIMT updates instead of tensor-core ones.
constexpr int kFp32Trsm = 256;
constexpr int kFp32Potrf = 2048;

__device__ __forceinline__ void put16(void* hi, void* lo, int64_t o, float v, int mode) {
  if (!hi) return;
  if (mode == 1) {
    reinterpret_cast<__nv_bfloat16*>(hi)[o] = __float2bfloat16_rn(v);
  } else {
    const __half h = __float2half_rn(v);
    reinterpret_cast<__half*>(hi)[o] = h;
    if (mode == 2) reinterpret_cast<__half*>(lo)[o] = __float2half_rn((v - __half2float(h)) * 2048.f);
  }
}

// Copies the nb x nb lower triangle of column-major L (ld ldl) into shared
// memory, element (i, j) at dst[i * si + j * sj]; zeros above the diagonal.
// Global reads are coalesced (i fastest) and issued eight per thread before
// the shared-memory stores, so the copy is not one memory latency per element.
__device__ __forceinline__ void stage_lower(int nb, const float* L, int64_t ldl, float* dst, int si, int sj) {
  const int total = nb * nb;
  const int T = blockDim.x;
  for (int base = threadIdx.x; base < total; base += 8 * T) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * T;
      const int i = e % nb, j = e / nb;
      v[u] = (e < total && j <= i) ? L[i + static_cast<int64_t>(j) * ldl] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * T;
      if (e < total) dst[(e % nb) * si + (e / nb) * sj] = v[u];
    }
  }
}

// Copies columns 0..nb-1 (rows 0..nb-1) of column-major L into shared memory
// column-major with stride `ldc` (a multiple of 4). float4 reads when L and ldl
// allow it; eight reads in flight per thread before the stores.
__device__ __forceinline__ void stage_cols(int nb, const float* L, int64_t ldl, float* dst, int ldc) {
  const int T = blockDim.x;
  const bool vec = (reinterpret_cast<uintptr_t>(L) % 16 == 0) && (ldl % 4 == 0) && (nb % 4 == 0);
  if (vec) {
    // (column, row quad) of element e: a shift when nq is a power of two (nb = 128: 32 quads), which
    // spares the integer divisions that otherwise dominate this copy
    const int nq = nb / 4, total = nq * nb;
    const bool pow2 = (nq & (nq - 1)) == 0;
    const int sh = __ffs(nq) - 1;
    for (int base = threadIdx.x; base < total; base += 8 * T) {
      float4 v[8];
      int off[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = base + u * T;
        const int c = pow2 ? e >> sh : e / nq, q = e - c * nq;
        off[u] = 4 * q + c * ldc;
        v[u] = e < total ? *reinterpret_cast<const float4*>(L + 4 * q + static_cast<int64_t>(c) * ldl)
                         : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (base + u * T < total) *reinterpret_cast<float4*>(dst + off[u]) = v[u];
    }
  } else {
    const int total = nb * nb;
    for (int base = threadIdx.x; base < total; base += 8 * T) {
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = base + u * T;
        v[u] = e < total ? L[e % nb + static_cast<int64_t>(e / nb) * ldl] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = base + u * T;
        if (e < total) dst[e % nb + (e / nb) * ldc] = v[u];
      }
    }
  }
}

// X L^T = B (right, lower, transposed), L nb x nb (nb <= 128), B m x nb.
// One CTA (256 threads) per R rows of B (R = 32 or 64), all of it parallel
// over rows and columns: the 32 x 32 diagonal blocks D_c of L are inverted
// once per CTA (warp c, lane = column of the inverse, forward substitution),
// then for each block column X_c = (B_c - X_<c L_c,<c^T) D_c^-T runs as two
// small shared-memory GEMMs in 2 x 4 register tiles: the product with D_c^-T,
// then the update of the columns after the block.
constexpr int LDL = 132;  // shared-memory stride of staged L (16-byte aligned)
constexpr int XS = 132;   // shared-memory row stride of the X tile

// Column `lane` of D^-1 into y (zeros above the diagonal) for the w x w lower-triangular diagonal block D
// starting at (cb, cb) of the column-major shared copy Lc (stride ldc), by forward substitution (one
// warp: lane = column). The Cholesky leaf and the triangular-solve leaf share it, so an inverse kept by
// the former is bit-identical to one the latter computes.
// Column k of D is read as float4 quads from the one holding row k (ldc and cb keep them 16-byte
// aligned): a quarter of the shared-memory loads of element-wise reads.
__device__ __forceinline__ void tri_block_inverse_col(const float* Lc, int ldc, int cb, int w, int lane,
                                                      float (&y)[32]) {
#pragma unroll
  for (int i = 0; i < 32; ++i) y[i] = (i == lane) ? 1.f : 0.f;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    if (k < w) {
      const float4* dq = reinterpret_cast<const float4*>(Lc + (cb + k) * ldc + cb);  // column k of D
      float d[32];
#pragma unroll
      for (int q = k / 4; q < 8; ++q) {
        const float4 v = dq[q];
        d[4 * q] = v.x;
        d[4 * q + 1] = v.y;
        d[4 * q + 2] = v.z;
        d[4 * q + 3] = v.w;
      }
      y[k] = y[k] / d[k];
#pragma unroll
      for (int i = k + 1; i < 32; ++i) y[i] -= d[i] * y[k];
    }
  }
}

// Table of the factor's 32 x 32 diagonal-block inverses (FP32), one slot per 32 columns: slot s holds
// D_s^-1 column-major, entry (i, j) at s * kDinvSlot + j * 32 + i, zeros outside the block.
constexpr int kDinvSlot = 32 * 32;

__global__ void __launch_bounds__(256) trsm_rlt_leaf(int m, int nb, int R, const float* __restrict__ L, int64_t ldl,
                                                     float* B, int64_t ldb, void* xh, void* xl, int64_t ldh,
                                                     int mode, const float* __restrict__ dinv) {
  griddep_wait();  // inputs come from the previous kernel in the stream
  griddep_launch();
  extern __shared__ __align__(16) float sm[];
  float* Lc = sm;             // L[j][l] at l*LDL + j; diagonal blocks replaced by their inverses
  float* Xs = sm + LDL * NB;  // X[r][c] at r*XS + c
  const int row0 = blockIdx.x * R;
  stage_cols(nb, L, ldl, Lc, LDL);
  {
    const int total = R * nb, shr = __ffs(R) - 1;  // R is 32 or 64
    for (int base = threadIdx.x; base < total; base += 8 * 256) {
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = base + u * 256;
        const int r = e & (R - 1), c = e >> shr;
        v[u] = (e < total && row0 + r < m) ? B[row0 + r + static_cast<int64_t>(c) * ldb] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = base + u * 256;
        if (e < total) Xs[(e & (R - 1)) * XS + (e >> shr)] = v[u];
      }
    }
  }
  __syncthreads();
  const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
  const int nblk = (nb + 31) / 32;
  if (dinv) {
    // the diagonal blocks' inverses, kept by the Cholesky leaf that factored L: whole 32 x 32 slots
    // (zeros outside each block), four rows per float4, every load of a thread in flight at once
    constexpr int kQ = 4 * kDinvSlot / 4 / 256;  // float4 per thread for four blocks
    float4 v[kQ];
#pragma unroll
    for (int u = 0; u < kQ; ++u) {
      const int q = threadIdx.x + u * 256;
      v[u] = q < nblk * kDinvSlot / 4 ? __ldcg(reinterpret_cast<const float4*>(dinv) + q)
                                      : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < kQ; ++u) {
      const int q = threadIdx.x + u * 256, e = 4 * q;
      const int blk = e / kDinvSlot, j = (e / 32) % 32, i = e % 32, cb = 32 * blk;
      if (q < nblk * kDinvSlot / 4) *reinterpret_cast<float4*>(&Lc[(cb + j) * LDL + cb + i]) = v[u];
    }
  } else {
    float y[32];
    const int cb = warp * 32, w = min(32, nb - cb);
    if (warp < nblk) tri_block_inverse_col(Lc, LDL, cb, w, lane, y);
    __syncthreads();  // every read of the diagonal blocks is done
    if (warp < nblk && lane < w) {
#pragma unroll
      for (int i = 0; i < 32; ++i)
        if (i < w) Lc[(cb + lane) * LDL + cb + i] = y[i];  // column `lane` of D^-1, zeros above the diagonal
    }
  }
  __syncthreads();
  for (int cb = 0; cb < nb; cb += 32) {
    const int w = min(32, nb - cb);
    // X_c <- X_c D_c^-T: out(r, j) = sum_i X[r][cb + i] Dinv[j][i]
    const bool act = threadIdx.x < (R / 2) * 8;
    const int ra = 2 * (threadIdx.x / 8), ja = 4 * (threadIdx.x % 8);
    float acc[2][4] = {};
    if (act) {
#pragma unroll 4
      for (int i = 0; i < w; ++i) {
        const float4 d = *reinterpret_cast<const float4*>(&Lc[(cb + i) * LDL + cb + ja]);
        const float x0 = Xs[ra * XS + cb + i], x1 = Xs[(ra + 1) * XS + cb + i];
        acc[0][0] += x0 * d.x; acc[0][1] += x0 * d.y; acc[0][2] += x0 * d.z; acc[0][3] += x0 * d.w;
        acc[1][0] += x1 * d.x; acc[1][1] += x1 * d.y; acc[1][2] += x1 * d.z; acc[1][3] += x1 * d.w;
      }
    }
    __syncthreads();
    if (act) {
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int row = row0 + ra + u;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const int j = ja + v;
          if (j < w) {
            Xs[(ra + u) * XS + cb + j] = acc[u][v];
            if (row < m) {
              const int64_t o = static_cast<int64_t>(cb + j);
              B[row + o * ldb] = acc[u][v];
              put16(xh, xl, row + o * ldh, acc[u][v], mode);
            }
          }
        }
      }
    }
    __syncthreads();
    // columns after the block: X[r][jj] -= sum_l X[r][cb + l] L[jj][cb + l]
    const int c1 = cb + w, W = nb - c1;
    if (W > 0) {
      const int nq = (W + 3) / 4, ntile = (R / 2) * nq;
      for (int q = threadIdx.x; q < ntile; q += 256) {
        const int r = 2 * (q / nq), jj = c1 + 4 * (q % nq);
        float a[2][4] = {};
#pragma unroll 8
        for (int l = 0; l < 32; ++l) {
          const float4 v = *reinterpret_cast<const float4*>(&Lc[(cb + l) * LDL + jj]);
          const float x0 = Xs[r * XS + cb + l], x1 = Xs[(r + 1) * XS + cb + l];
          a[0][0] += x0 * v.x; a[0][1] += x0 * v.y; a[0][2] += x0 * v.z; a[0][3] += x0 * v.w;
          a[1][0] += x1 * v.x; a[1][1] += x1 * v.y; a[1][2] += x1 * v.z; a[1][3] += x1 * v.w;
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v)
            if (jj + v < nb) Xs[(r + u) * XS + jj + v] -= a[u][v];
      }
    }
    __syncthreads();
  }
}

// L X = B (left, lower, no transpose), L nb x nb (nb <= 128), B nb x n. One
// warp per column of B, eight columns per CTA; lane l holds rows l, l+32,
// l+64, l+96. Right-looking: x_k is broadcast from its owner lane and every
// lane updates its rows below k. L is staged column-major (stride 129).
__global__ void __launch_bounds__(256) trsm_lln_leaf(int nb, int n, const float* __restrict__ L, int64_t ldl, float* B,
                                                     int64_t ldb, void* xh, void* xl, int64_t ldh, int mode) {
  griddep_wait();  // inputs come from the previous kernel in the stream
  griddep_launch();
  extern __shared__ __align__(16) float sm[];
  float* Lc = sm;  // L[i][k] at i + k*129
  stage_lower(nb, L, ldl, Lc, 1, 129);
  __syncthreads();
  const int lane = threadIdx.x % 32;
  const int c = blockIdx.x * 8 + threadIdx.x / 32;
  if (c >= n) return;
  float b[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = lane + 32 * q;
    b[q] = r < nb ? B[r + static_cast<int64_t>(c) * ldb] : 0.f;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    for (int kk = 0; kk < 32; ++kk) {
      const int k = 32 * q + kk;
      if (k >= nb) break;
      const float xk = __shfl_sync(0xffffffffu, b[q], kk) / Lc[k + k * 129];
      if (lane == kk) b[q] = xk;
#pragma unroll
      for (int q2 = q; q2 < 4; ++q2) {
        const int r = lane + 32 * q2;
        if (r > k && r < nb) b[q2] -= Lc[r + k * 129] * xk;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = lane + 32 * q;
    if (r < nb) {
      B[r + static_cast<int64_t>(c) * ldb] = b[q];
      put16(xh, xl, r + static_cast<int64_t>(c) * ldh, b[q], mode);
    }
  }
}

// L^T X = B (left, lower, transposed), L nb x nb (nb <= 128), B nb x n:
// backward substitution, one warp per column as above; L is staged row-major
// (stride 129) so that row k of L, which multiplies x_k, is contiguous.
__global__ void __launch_bounds__(256) trsm_llt_leaf(int nb, int n, const float* __restrict__ L, int64_t ldl, float* B,
                                                     int64_t ldb) {
  griddep_wait();  // inputs come from the previous kernel in the stream
  griddep_launch();
  extern __shared__ __align__(16) float sm[];
  float* Lr = sm;  // L[k][i] at k*129 + i
  stage_lower(nb, L, ldl, Lr, 129, 1);
  __syncthreads();
  const int lane = threadIdx.x % 32;
  const int c = blockIdx.x * 8 + threadIdx.x / 32;
  if (c >= n) return;
  float b[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = lane + 32 * q;
    b[q] = r < nb ? B[r + static_cast<int64_t>(c) * ldb] : 0.f;
  }
#pragma unroll
  for (int q = 3; q >= 0; --q) {
    for (int kk = 31; kk >= 0; --kk) {
      const int k = 32 * q + kk;
      if (k >= nb) continue;
      const float xk = __shfl_sync(0xffffffffu, b[q], kk) / Lr[k * 129 + k];
      if (lane == kk) b[q] = xk;
#pragma unroll
      for (int q2 = 0; q2 <= q; ++q2) {
        const int r = lane + 32 * q2;
        if (r < k) b[q2] -= Lr[k * 129 + r] * xk;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = lane + 32 * q;
    if (r < nb) B[r + static_cast<int64_t>(c) * ldb] = b[q];
  }
}

// C = L B (left, lower), L nb x nb (nb <= 128), B nb x n, C nb x n. One CTA
// per 64 columns; each thread accumulates 8 rows x 4 columns... of its share.
__global__ void __launch_bounds__(256) trmm_leaf(int nb, int n, const float* __restrict__ L, int64_t ldl,
                                                 const float* __restrict__ B, int64_t ldb, float* C, int64_t ldc) {
  griddep_wait();  // inputs come from the previous kernel in the stream
  griddep_launch();
  extern __shared__ float sm[];
  float* Ls = sm;             // [i][k]
  float* Bs = sm + NB * 129;  // [k][c] at k*65 + c
  const int c0 = blockIdx.x * 64;
  stage_lower(nb, L, ldl, Ls, 129, 1);
  for (int base = threadIdx.x; base < nb * 64; base += 8 * 256) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + 256 * u;
      const int k = e % nb, c = e / nb;
      v[u] = (e < nb * 64 && c0 + c < n) ? B[k + static_cast<int64_t>(c0 + c) * ldb] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + 256 * u;
      if (e < nb * 64) Bs[(e % nb) * 65 + e / nb] = v[u];
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nb * 64; e += 256) {
    const int i = e % nb, c = e / nb;
    if (c0 + c >= n) continue;
    float acc = 0.f;
    for (int k = 0; k <= i; ++k) acc += Ls[i * 129 + k] * Bs[k * 65 + c];
    C[i + static_cast<int64_t>(c0 + c) * ldc] = acc;
  }
}

// Inverse of the nb x nb lower-triangular L in shared memory (nb <= 128;
// L[i][j] at Lc[j * ldc + i], ldc a multiple of 4) into V (same layout, zeros
// above the diagonal). 32 x 32 blocks: warp c inverts diagonal block c by
// forward substitution, lane = column of the inverse; then, by growing
// distance d = I - J from the diagonal, T_J = sum_{K=J}^{I-1} L_IK V_KJ and
// V_IJ = -V_II T_J, the blocks of one distance in parallel, 64 threads per
// block in 4 x 4 register tiles (T: 3 x 32 x 36 floats of scratch). Rows and
// columns of V beyond nb are zero. All threads call it.
__device__ void tri_inverse_smem(int nb, const float* Lc, int ldc, float* V, float* T) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nblk = (nb + 31) / 32, np = nblk * 32;
  for (int e = threadIdx.x; e < np * np; e += blockDim.x) V[(e / np) * ldc + e % np] = 0.f;
  __syncthreads();
  if (warp < nblk) {
    const int cb = warp * 32, w = min(32, nb - cb);
    float y[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) y[i] = (i == lane) ? 1.f : 0.f;
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      if (k < w) {
        const float* dcol = Lc + (cb + k) * ldc + cb;  // column k of the diagonal block
        y[k] = y[k] / dcol[k];
#pragma unroll
        for (int i = k + 1; i < 32; ++i)
          if (i < w) y[i] -= dcol[i] * y[k];
      }
    }
    if (lane < w) {
#pragma unroll
      for (int i = 0; i < 32; ++i)
        if (i < w) V[(cb + lane) * ldc + cb + i] = y[i];
    }
  }
  __syncthreads();
  const int blk = threadIdx.x / 64, t = threadIdx.x % 64;
  const int r0 = 4 * (t % 8), c0 = 4 * (t / 8);  // this thread's 4 x 4 tile inside a 32 x 32 block
  for (int d = 1; d < nblk; ++d) {
    const bool act = blk < nblk - d;
    const int J = blk, I = blk + d;
    if (act) {
      float acc[4][4] = {};
      const int rowI = I * 32 + r0;
#pragma unroll 4
      for (int k = J * 32; k < I * 32; ++k) {
        // rows of L at or beyond nb hold whatever the caller's staging left there: masked, so that
        // T's rows there are zero (they meet zero columns of V_II below)
        const float4 a = *reinterpret_cast<const float4*>(&Lc[k * ldc + rowI]);
        const float av[4] = {rowI < nb ? a.x : 0.f, rowI + 1 < nb ? a.y : 0.f, rowI + 2 < nb ? a.z : 0.f,
                             rowI + 3 < nb ? a.w : 0.f};
        float bv[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) bv[v] = V[(J * 32 + c0 + v) * ldc + k];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        *reinterpret_cast<float4*>(&T[J * 1152 + (r0 + u) * 36 + c0]) =
            make_float4(acc[u][0], acc[u][1], acc[u][2], acc[u][3]);
    }
    __syncthreads();
    if (act) {
      float acc[4][4] = {};
      const int rowI = I * 32 + r0;
#pragma unroll 4
      for (int k = 0; k < 32; ++k) {
        const float4 a = *reinterpret_cast<const float4*>(&V[(I * 32 + k) * ldc + rowI]);
        const float4 b = *reinterpret_cast<const float4*>(&T[J * 1152 + k * 36 + c0]);
        const float av[4] = {a.x, a.y, a.z, a.w};
        const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
      }
#pragma unroll
      for (int v = 0; v < 4; ++v)
        *reinterpret_cast<float4*>(&V[(J * 32 + c0 + v) * ldc + rowI]) =
            make_float4(-acc[0][v], -acc[1][v], -acc[2][v], -acc[3][v]);
    }
    __syncthreads();
  }
  // entries of the padding (rows or columns >= nb) must stay zero for the caller
  for (int e = threadIdx.x; e < np * np; e += blockDim.x) {
    const int i = e % np, j = e / np;
    if (i >= nb || j >= nb) V[j * ldc + i] = 0.f;
  }
  __syncthreads();
}

// Lower Cholesky of an nb x nb block (nb <= 128) in one CTA, in shared memory
// (column-major, stride LDL), right-looking over 32-column blocks with a
// look-ahead of one block. Warp 0 factors the 32 x 32 diagonal block with the
// compact register-window Cholesky (dense_dev.cuh; pivots d * rsqrt(d)) and
// publishes its pivots eight at a time on named barriers; behind it, warps
// 1..7 first apply the previous block's deferred update to the columns right
// of this block, then solve the rows below this block (x R = a, eight columns
// per published pivot group). After the block, the whole CTA updates only the
// next block's columns, so the next Cholesky can start; the rest of the
// update waits for it. Every entry receives the blocks' updates in block
// order, each a 4 x 4-tiled sum over the block's 32 columns. A non-positive
// (or NaN) pivot sets DEV_NUMERIC; the factorisation continues (with pivot 1)
// so the kernel always finishes.
struct PotrfSmem {
  float G[32 * 33];   // the diagonal block, row-major
  float Rc[32 * RCS]; // its factor, column-major R = L^T
  float rinv[32];
  int ok;
};

// Named barriers of potrf_leaf: one per pivot group of eight (kPotrfPub + g, counting warps 0..6:
// warp 0 arrives, warps 1..6 wait; warp 7 inverts the previous diagonal block meanwhile).
constexpr int kPotrfPub = 1;  // ids 1 .. 4
constexpr int kPotrfPubCount = 7 * 32;

// A[i][j] -= sum_{l < kb} A[i][k0 + l] A[j][k0 + l] for the lower-triangle entries j in [j0, j1), i in
// [j, nb), in 4 x 4 tiles (j0 a multiple of 4), by threads t (of nthr) of the CTA.
__device__ __forceinline__ void potrf_syrk(float* Ac, int nb, int k0, int kb, int j0, int j1, int t, int nthr) {
  const int ncol = (j1 - j0 + 3) / 4;
  // column tile c spans columns j0 + 4c .. + 3 and row tiles from row j0 + 4c to nb
  int total = 0;
  for (int c = 0; c < ncol; ++c) total += (nb - (j0 + 4 * c) + 3) / 4;
  for (int q = t; q < total; q += nthr) {
    int c = 0, rem = q;
    for (;; ++c) {
      const int nr = (nb - (j0 + 4 * c) + 3) / 4;
      if (rem < nr) break;
      rem -= nr;
    }
    const int c0 = j0 + 4 * c, i0 = c0 + 4 * rem;
    float acc[4][4] = {};
#pragma unroll 8
    for (int l = 0; l < kb; ++l) {
      const float4 a = *reinterpret_cast<const float4*>(&Ac[(k0 + l) * LDL + i0]);
      const float4 b = *reinterpret_cast<const float4*>(&Ac[(k0 + l) * LDL + c0]);
      const float av[4] = {a.x, a.y, a.z, a.w};
      const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int i = i0 + u, j = c0 + v;
        if (i < nb && j < j1 && j <= i) Ac[j * LDL + i] -= acc[u][v];
      }
  }
}

// A[i][j] -= sum_{l < kw} A[i][kc + l] A[j][kc + l] for the lower entries of the w x w diagonal block at
// (j0, j0), w <= 32, j0 a multiple of 4: lane i of warp g computes row i, columns 4 g .. 4 g + 3
// (256 threads; no barrier inside).
__device__ __forceinline__ void potrf_diag_update(float* Ac, int kc, int kw, int j0, int w) {
  const int i = threadIdx.x & 31, g = threadIdx.x >> 5;
  if (4 * g >= w) return;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
  for (int l = 0; l < kw; ++l) {
    const float a = i < w ? Ac[(kc + l) * LDL + j0 + i] : 0.f;
    const float4 b = *reinterpret_cast<const float4*>(&Ac[(kc + l) * LDL + j0 + 4 * g]);
    acc[0] = fmaf(a, b.x, acc[0]);
    acc[1] = fmaf(a, b.y, acc[1]);
    acc[2] = fmaf(a, b.z, acc[2]);
    acc[3] = fmaf(a, b.w, acc[3]);
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int j = 4 * g + v;
    if (i < w && j < w && j <= i) Ac[(j0 + j) * LDL + j0 + i] -= acc[v];
  }
}

// Row r: A[r][j0 + j] -= sum_{l < kw} A[r][kc + l] A[j0 + j][kc + l] for j < w (w <= 32, j0 a multiple of 4).
__device__ __forceinline__ void potrf_row_update(float* Ac, int r, int kc, int kw, int j0, int w) {
  float acc[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) acc[j] = 0.f;
#pragma unroll 2
  for (int l = 0; l < kw; ++l) {
    const float a = Ac[(kc + l) * LDL + r];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float4 b = *reinterpret_cast<const float4*>(&Ac[(kc + l) * LDL + j0 + 4 * q]);
      acc[4 * q] = fmaf(a, b.x, acc[4 * q]);
      acc[4 * q + 1] = fmaf(a, b.y, acc[4 * q + 1]);
      acc[4 * q + 2] = fmaf(a, b.z, acc[4 * q + 2]);
      acc[4 * q + 3] = fmaf(a, b.w, acc[4 * q + 3]);
    }
  }
#pragma unroll
  for (int j = 0; j < 32; ++j)
    if (j < w) Ac[(j0 + j) * LDL + r] -= acc[j];
}

// The w x w diagonal block at (cb, cb) of Ac, inverted by one warp into the table slot `out`.
__device__ __forceinline__ void potrf_keep_inverse(const float* Ac, int cb, int w, float* out) {
  const int lane = threadIdx.x & 31;
  float y[32];
  tri_block_inverse_col(Ac, LDL, cb, w, lane, y);
#pragma unroll
  for (int i = 0; i < 32; ++i) out[lane * 32 + i] = (lane < w && i < w) ? y[i] : 0.f;
}

__global__ void __launch_bounds__(256, 1) potrf_leaf(int nb, float* A, int64_t lda, int* status, float* dinv) {
  griddep_wait();  // inputs come from the previous kernel in the stream
  griddep_launch();
  extern __shared__ __align__(16) float sm[];
  float* Ac = sm;  // A[i][j] at j*LDL + i (lower triangle used)
  PotrfSmem& ps = *reinterpret_cast<PotrfSmem*>(sm + LDL * NB);
  stage_cols(nb, A, lda, Ac, LDL);
  __syncthreads();
  const int tid = threadIdx.x;
  bool bad = false;
  for (int k0 = 0; k0 < nb; k0 += 32) {
    const int kb = min(32, nb - k0);
    const int t0 = k0 + kb;  // first row below the block
    for (int e = tid; e < 32 * 32; e += blockDim.x) {
      const int i = e / 32, j = e % 32;
      ps.G[i * 33 + j] = (i < kb && j < kb && j <= i) ? Ac[(k0 + j) * LDL + k0 + i] : 0.f;
    }
    __syncthreads();
    if (tid < 32) {
      chol_upper(ps.G, kb, ps.Rc, ps.rinv, false, &ps.ok, 0.f, kPotrfPub, kPotrfPubCount);
    } else {
      const int ct = tid - 32, nct = static_cast<int>(blockDim.x) - 32;
      // warp 7: the previous diagonal block's inverse into the table, for the triangular solves
      if (tid >= kPotrfPubCount && k0 > 0 && dinv)
        potrf_keep_inverse(Ac, k0 - 32, 32, dinv + (k0 / 32 - 1) * kDinvSlot);
      // the previous block's update of the columns right of this block (deferred to this phase; it
      // touches neither this block's columns, which the solve below works on, nor the copy in G)
      if (k0 > 0 && t0 < nb) potrf_syrk(Ac, nb, k0 - 32, 32, t0, nb, ct, nct);
      // rows below the block: x R = a with R = L_D^T, eight columns per published pivot group (warps 1..6);
      // first each row's share of the previous block's update of this block's columns (the end of the
      // previous phase updated only the diagonal block)
      if (tid < kPotrfPubCount) {
        const int nsv = kPotrfPubCount - 32;
        if (k0 > 0)
          for (int r = t0 + ct; r < nb; r += nsv) potrf_row_update(Ac, r, k0 - 32, 32, k0, kb);
        for (int b = 0; b < kb; b += 8) {
          asm volatile("bar.sync %0, %1;" ::"r"(kPotrfPub + b / 8), "r"(kPotrfPubCount) : "memory");
          for (int r = t0 + ct; r < nb; r += nsv) rows_solve_group(Ac + k0 * LDL, LDL, kb, r, ps.Rc, ps.rinv, b);
        }
      }
    }
    __syncthreads();
    if (!ps.ok) bad = true;
    // the factor back into the block: L[i][j] = R[j][i] = Rc[i * RCS + j]
    for (int e = tid; e < 32 * 32; e += blockDim.x) {
      const int i = e & 31, j = e >> 5;
      if (j <= i && i < kb) Ac[(k0 + j) * LDL + k0 + i] = ps.Rc[i * RCS + j];
    }
    // this block's update of the next diagonal block only; the rows below it follow in the next phase
    // (each by the thread that solves it), the columns further right in the phase after
    // (it reads only rows below this diagonal block, which the write-back above does not touch)
    if (t0 < nb) potrf_diag_update(Ac, k0, kb, t0, min(32, nb - t0));
    __syncthreads();
  }
  if (bad && tid == 0) report(status, DEV_NUMERIC);
  // the last diagonal block's inverse (warp 7), beside the store of the factor
  const int klast = (nb - 1) / 32 * 32;
  if (tid >= kPotrfPubCount && dinv) potrf_keep_inverse(Ac, klast, nb - klast, dinv + (klast / 32) * kDinvSlot);
  // the factor back to A: a column per warp, lanes along its rows on and below the diagonal
  for (int j = tid / 32; j < nb; j += blockDim.x / 32)
    for (int i = j + (tid & 31); i < nb; i += 32) A[i + static_cast<int64_t>(j) * lda] = Ac[j * LDL + i];
}

// Inverses of diagonal blocks of a lower-triangular factor, one CTA per block
// (block i: columns [col[i], col[i] + w[i]) of L, w[i] <= 128), written as hi +
// lo 16-bit pairs (ld 128) to slot col[i] / 64 of the tables.
constexpr int kMaxInvBlocks = 160;
struct InvBlocks {
  int n;
  int col[kMaxInvBlocks];
  int w[kMaxInvBlocks];
};

__global__ void __launch_bounds__(256) trtri_blocks_kernel(const float* __restrict__ L, int64_t ldl, InvBlocks blocks,
                                                           __half* vh_tab, __half* vl_tab) {
  griddep_wait();  // inputs come from the previous kernel in the stream
  griddep_launch();
  extern __shared__ __align__(16) float sm[];
  float* Lc = sm;
  float* V = sm + LDL * NB;
  float* T = V + LDL * NB;
  const int c = blocks.col[blockIdx.x], nb = blocks.w[blockIdx.x];
  stage_cols(nb, L + c + static_cast<int64_t>(c) * ldl, ldl, Lc, LDL);
  __syncthreads();
  tri_inverse_smem(nb, Lc, LDL, V, T);
  __half* vh = vh_tab + static_cast<int64_t>(c / 64) * (128 * 128);
  __half* vl = vl_tab + static_cast<int64_t>(c / 64) * (128 * 128);
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e % nb, j = e / nb;
    const float v = V[j * LDL + i];
    const __half h = __float2half_rn(v);
    vh[i + j * 128] = h;
    vl[i + j * 128] = __float2half_rn((v - __half2float(h)) * 2048.f);
  }
}

// Inverses of 256-column diagonal blocks from the inverses of their two 128-column halves, one CTA per
// block: for L = [L11 0; L21 L22] (block i: columns [col[i], col[i] + 256), col[i] a multiple of 128),
// L^-1 = [I1 0; -I2 L21 I1 I2] with I1 = L11^-1 and I2 = L22^-1 read from the 128-column tables (slots
// col / 64 and col / 64 + 2). P = L21 I1 and X21 = -I2 P are two 128 x 128 x 128 FP32 products in shared
// memory; the whole inverse goes out as a hi + lo 16-bit pair (ld 256) to slot col[i] / 128.
constexpr int kMaxInvPairs = 80;
struct InvPairs {
  int n;
  int col[kMaxInvPairs];
};

// acc[u][v] += sum_k A[k][i] B[k][j], i = ty + 16 u, j = tx + 16 v: Acm holds A column-major (A[i][k] at
// k * LDL + i), Brm holds B row-major (B[k][j] at k * LDL + j); 256 threads, 8 x 8 outputs each.
__device__ __forceinline__ void smem_mm128(const float* Acm, const float* Brm, float (&acc)[8][8]) {
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
#pragma unroll 2
  for (int k = 0; k < NB; ++k) {
    float a[8], bv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) a[u] = Acm[k * LDL + ty + 16 * u];
#pragma unroll
    for (int v = 0; v < 8; ++v) bv[v] = Brm[k * LDL + tx + 16 * v];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(a[u], bv[v], acc[u][v]);
  }
}

__device__ __forceinline__ float unsplit(const __half* hi, const __half* lo, int64_t e) {
  return __half2float(hi[e]) + __half2float(lo[e]) * (1.f / 2048.f);
}

__global__ void __launch_bounds__(256, 1) inv256_kernel(const float* __restrict__ L, int64_t ldl, InvPairs pairs,
                                                        const __half* __restrict__ vh_tab,
                                                        const __half* __restrict__ vl_tab, __half* wh_tab,
                                                        __half* wl_tab) {
  griddep_wait();  // inputs come from the previous kernel in the stream
  griddep_launch();
  extern __shared__ __align__(16) float sm[];
  float* S0 = sm;                // L21 (column-major), then I2 (column-major)
  float* S1 = sm + LDL * NB;     // I1 (row-major)
  float* S2 = S1 + LDL * NB;     // P = L21 I1 (row-major)
  const int c = pairs.col[blockIdx.x];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const __half* i1h = vh_tab + static_cast<int64_t>(c / 64) * (128 * 128);
  const __half* i1l = vl_tab + static_cast<int64_t>(c / 64) * (128 * 128);
  const __half* i2h = i1h + 2 * (128 * 128);  // slot c / 64 + 2: the block at column c + 128
  const __half* i2l = i1l + 2 * (128 * 128);
  __half* wh = wh_tab + static_cast<int64_t>(c / 128) * (256 * 256);
  __half* wl = wl_tab + static_cast<int64_t>(c / 128) * (256 * 256);
  stage_cols(NB, L + (c + NB) + static_cast<int64_t>(c) * ldl, ldl, S0, LDL);
  // I1 row-major: entry (k, j) of the table (column-major, ld 128) at k * LDL + j
  for (int e = tid; e < NB * NB; e += 256) {
    const int k = e & (NB - 1), j = e >> 7;
    S1[k * LDL + j] = unsplit(i1h, i1l, e);
  }
  // the diagonal blocks and the zero upper-right block of the 256 x 256 inverse, straight from the tables
  for (int e = tid; e < NB * NB; e += 256) {
    const int i = e & (NB - 1), j = e >> 7;
    wh[i + j * 256] = i1h[e];
    wl[i + j * 256] = i1l[e];
    wh[(NB + i) + (NB + j) * 256] = i2h[e];
    wl[(NB + i) + (NB + j) * 256] = i2l[e];
    wh[i + (NB + j) * 256] = __float2half_rn(0.f);
    wl[i + (NB + j) * 256] = __float2half_rn(0.f);
  }
  __syncthreads();
  float acc[8][8];
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
  smem_mm128(S0, S1, acc);  // P = L21 I1
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) S2[(ty + 16 * u) * LDL + tx + 16 * v] = acc[u][v];
  __syncthreads();
  // I2 column-major into S0 (L21 is no longer needed)
  for (int e = tid; e < NB * NB; e += 256) {
    const int i = e & (NB - 1), k = e >> 7;
    S0[k * LDL + i] = unsplit(i2h, i2l, e);
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
  smem_mm128(S0, S2, acc);  // I2 P
#pragma unroll
  for (int u = 0; u < 8; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const int i = ty + 16 * u, j = tx + 16 * v;
      const float x = -acc[u][v];
      const __half h = __float2half_rn(x);
      wh[(NB + i) + j * 256] = h;
      wl[(NB + i) + j * 256] = __float2half_rn((x - __half2float(h)) * 2048.f);
    }
}

constexpr size_t kPotrfLeafSmem = (LDL * NB) * sizeof(float) + (sizeof(PotrfSmem) + 15) / 16 * 16;
constexpr size_t kTrtriSmem = (2 * LDL * NB + 3 * 1152) * sizeof(float);
static_assert(kTrtriSmem <= 227 * 1024, "block inverse shared memory");
constexpr size_t kInv256Smem = 3 * LDL * NB * sizeof(float);
static_assert(kInv256Smem <= 227 * 1024, "256-column inverse shared memory");

inline int mode_of(int prec) { return prec == LATER_PREC_BF16 ? 1 : (prec == LATER_PREC_SPLIT3 ? 2 : 0); }

// Splits n in half, rounded to a multiple of 64 (keeps 16-bit row offsets
// 16-byte aligned for the tensor maps).
inline int half64(int n) { return std::max(64, static_cast<int>(round_up(n / 2, 64))); }

bool smem_attr(const void* fn, size_t bytes) {
  static bool done[8][64] = {};
  static const void* fns[8] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  int slot = 0;
  for (; slot < 8; ++slot)
    if (fns[slot] == fn || fns[slot] == nullptr) break;
  if (slot == 8 || dev >= 64) return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          static_cast<int>(bytes)) == cudaSuccess;
  fns[slot] = fn;
  if (!done[slot][dev]) {
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)) != cudaSuccess)
      return false;
    done[slot][dev] = true;
  }
  return true;
}

struct B3 {
  cudaStream_t st;
  Options o;
  Arena* ws = nullptr;  // FP32 scratch for SIMT partial products (optional)
  char* h;      // 16-bit scratch (hwork) cursor
  size_t hcap;  // bytes
  Scratch sc;   // split-K scratch
  // Cholesky only: the updates below the FP32 thresholds run as SPLIT3 tensor-core products (FP32-level)
  // instead of SIMT FP32 ones, and, when inv_hi is set, the triangular solves against a diagonal block of
  // the factor are products with that block's inverse, kept by the Cholesky leaves at slot col / 64.
  bool tc_small = false;
  bool leaf_gemm = false;
  __half* inv_hi = nullptr;
  __half* inv_lo = nullptr;
  std::vector<char>* inv_done = nullptr;  // per slot: inverse already in the table
  // Cholesky only: the factor's 32 x 32 diagonal-block inverses (FP32), kept by the Cholesky leaves for the
  // triangular-solve leaves (slot = factor column / 32)
  float* dinv = nullptr;
  // Cholesky only: blocks of at most kFp32Potrf columns are factored by the blocked loop (potrf_blocked)
  // rather than by the recursion
  bool blocked = false;
  // Cholesky only: inverses of 256-column diagonal blocks (hi + lo, ld 256, slot = col / 128); a solve
  // against such a block whose inverse is present is one product instead of two and an update between
  __half* inv2_hi = nullptr;
  __half* inv2_lo = nullptr;
  std::vector<char>* inv2_done = nullptr;
};

// LATER_POTRF_BLOCKED=0 factors the blocks below kFp32Potrf columns by the recursion instead (comparison runs)
bool potrf_blocked_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("LATER_POTRF_BLOCKED");
    return !(e && e[0] == '0');
  }();
  return on;
}

// LATER_POTRF_INV256=0 keeps the solves against 128-column inverses only (comparison runs)
bool inv2_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("LATER_POTRF_INV256");
    return !(e && e[0] == '0');
  }();
  return on;
}

// Solves with at least this many rows use the diagonal block's inverse (its
// one-off inversion is then cheaper than the substitution it replaces).
constexpr int kInvMinRows = 2048;

constexpr int64_t kInvSlot = 128 * 128;  // 16-bit elements per inverse block (ld 128)
inline int64_t inv_slots(int n) { return (n + 63) / 64; }
constexpr int64_t kInv2Slot = 256 * 256;  // 16-bit elements per 256-column inverse (ld 256)
inline int64_t inv2_slots(int n) { return (n + 127) / 128; }
inline int64_t dinv_slots(int n) { return (n + 31) / 32; }

// Takes `elems` 16-bit elements from the hwork scratch (256-byte aligned).
char* take16(B3& b, int64_t elems, size_t* mark) {
  const uintptr_t p = (reinterpret_cast<uintptr_t>(b.h) + 255) & ~uintptr_t(255);
  const size_t used = p - reinterpret_cast<uintptr_t>(b.h);
  const size_t need = used + static_cast<size_t>(elems) * 2 * (b.o.prec == LATER_PREC_SPLIT3 ? 2 : 1);
  if (need > b.hcap) return nullptr;
  *mark = need;
  return reinterpret_cast<char*>(p);
}

// 16-bit copy of an m x n FP32 block into the scratch (hi, and lo for SPLIT3).
later_status_t copy16(B3& b, int m, int n, const float* X, int64_t ldx, Op16* out, size_t* used) {
  const int64_t ld = round_up(m, 8);
  size_t mark = 0;
  char* p = take16(b, ld * n, &mark);
  if (!p) return LATER_ERR_WORKSPACE;
  out->hi = p;
  out->lo = b.o.prec == LATER_PREC_SPLIT3 ? p + ld * n * 2 : nullptr;
  out->ld = ld;
  *used = mark;
  return convert16(b.st, m, n, X, ldx, const_cast<void*>(out->hi), const_cast<void*>(out->lo), ld, b.o.prec);
}

later_status_t gemm(B3& b, char ta, char tb, int M, int N, int K, float alpha, const Op16& A, const Op16& Bm,
                    float beta, float* C, int64_t ldc, void* dh = nullptr, void* dl = nullptr, int64_t ldh = 0,
                    int lower = 0) {
  GemmCall g;
  g.ta = ta;
  g.tb = tb;
  g.M = M;
  g.N = N;
  g.K = K;
  g.A = A;
  g.B = Bm;
  g.alpha = alpha;
  g.beta = beta;
  g.out.C = C;
  g.out.ldc = ldc;
  g.out.D = C;
  g.out.ldd = ldc;
  g.out.Dh = dh;
  g.out.Dl = dl;
  g.out.ldh = ldh;
  g.out.lower = lower;
  g.prec = b.o.prec;
  g.out_prec = b.o.prec;
  return tc_gemm(g, b.sc, b.st, b.o.budget);
}

// -------------------------------------------------------------- recursions
// X L^T = B, L n x n, B m x n. X's 16-bit copy goes to (xh, ldh) (columns as B).
// Updates are FP32 while n <= fp32_lim, tensor-core above.
later_status_t trsm_rlt(B3& b, int m, int n, const float* L, int64_t ldl, float* B, int64_t ldb, char* xh, char* xl,
                        int64_t ldh, int fp32_lim = kFp32Trsm, int64_t col = -1) {
  if (n == 2 * NB && b.leaf_gemm && b.inv2_hi && col >= 0 && col % NB == 0 && m >= kInvMinRows && b.inv2_done &&
      (*b.inv2_done)[col / NB]) {
    // X = B L^-T against the 256-column block's inverse: one SPLIT3 product replaces the two half-block
    // products and the update between them
    B3 sub = b;
    sub.o.prec = LATER_PREC_SPLIT3;
    Op16 bb;
    size_t used = 0;
    LATER_CHECK(copy16(sub, m, n, B, ldb, &bb, &used));
    sub.h += used;
    sub.hcap -= used;
    const Op16 winv{b.inv2_hi + (col / NB) * kInv2Slot, b.inv2_lo + (col / NB) * kInv2Slot, 2 * NB};
    GemmCall g;
    g.ta = 'N';
    g.tb = 'T';
    g.M = m;
    g.N = n;
    g.K = n;
    g.A = bb;
    g.B = winv;
    g.out.D = B;
    g.out.ldd = ldb;
    g.out.Dh = xh;
    g.out.Dl = xl;
    g.out.ldh = ldh;
    g.prec = LATER_PREC_SPLIT3;
    g.out_prec = xl ? LATER_PREC_SPLIT3 : b.o.prec;
    return tc_gemm(g, sub.sc, b.st, b.o.budget);
  }
  if (n <= NB && b.leaf_gemm && b.inv_hi && col >= 0 && m >= kInvMinRows && b.inv_done &&
      (*b.inv_done)[col / 64]) {
    // X = B L^-T as one SPLIT3 tensor-core product with the block's inverse (FP32-level operands)
    B3 sub = b;
    sub.o.prec = LATER_PREC_SPLIT3;
    Op16 bb;
    size_t used = 0;
    LATER_CHECK(copy16(sub, m, n, B, ldb, &bb, &used));
    sub.h += used;
    sub.hcap -= used;
    const Op16 vinv{b.inv_hi + (col / 64) * kInvSlot, b.inv_lo + (col / 64) * kInvSlot, 128};
    GemmCall g;
    g.ta = 'N';
    g.tb = 'T';
    g.M = m;
    g.N = n;
    g.K = n;
    g.A = bb;
    g.B = vinv;
    g.out.D = B;
    g.out.ldd = ldb;
    g.out.Dh = xh;
    g.out.Dl = xl;
    g.out.ldh = ldh;
    g.prec = LATER_PREC_SPLIT3;
    g.out_prec = xl ? LATER_PREC_SPLIT3 : b.o.prec;  // with xl: X's copy as a hi + lo pair
    return tc_gemm(g, sub.sc, b.st, b.o.budget);
  }
  if (n <= NB) {
    const size_t smem = (LDL * NB + 64 * XS) * sizeof(float);
    if (!smem_attr(reinterpret_cast<const void*>(trsm_rlt_leaf), smem)) return LATER_ERR_CUDA;
    TraceScope tr(b.st, TRACE_OTHER);
    // 64 rows per CTA while that still gives two CTAs per SM, else 32
    const int R = (m + 63) / 64 >= 2 * num_sms() ? 64 : 32;
    const float* dinv = (b.dinv && col >= 0) ? b.dinv + (col / 32) * kDinvSlot : nullptr;
    LATER_CHECK_CUDA(launch_pdl(trsm_rlt_leaf, dim3((m + R - 1) / R), dim3(256), smem, b.st, m, n, R, L, ldl, B, ldb,
                                xh, xl, ldh, xl ? 2 : mode_of(b.o.prec), dinv));
    note_launch();
    return cuda_status(cudaGetLastError());
  }
  const int n1 = half64(n), n2 = n - n1;
  LATER_CHECK(trsm_rlt(b, m, n1, L, ldl, B, ldb, xh, xl, ldh, fp32_lim, col));
  // B2 -= X1 L21^T   (L21 = L[n1:, :n1], n2 x n1)
  if (n <= fp32_lim && b.tc_small) {
    // FP32-level: both operands freshly split into SPLIT3 pairs
    B3 sub = b;
    sub.o.prec = LATER_PREC_SPLIT3;
    Op16 x1{xh, xl, ldh}, l21;  // X1's hi + lo pair, written by its solve, when the caller keeps one
    size_t used = 0;
    if (!xh || !xl) {
      LATER_CHECK(copy16(sub, m, n1, B, ldb, &x1, &used));
      sub.h += used;
      sub.hcap -= used;
    }
    LATER_CHECK(copy16(sub, n2, n1, L + n1, ldl, &l21, &used));
    sub.h += used;
    sub.hcap -= used;
    LATER_CHECK(gemm(sub, 'N', 'T', m, n2, n1, -1.f, x1, l21, 1.f, B + n1 * ldb, ldb));
  } else if (n <= fp32_lim) {
    LATER_CHECK(simt_gemm_acc(b.st, m, n1, n2, -1.f, B, ldb, L + n1, ldl, 1, 0, B + n1 * ldb, ldb));
  } else {
    B3 sub = b;
    Op16 l21;
    size_t used = 0;
    LATER_CHECK(copy16(sub, n2, n1, L + n1, ldl, &l21, &used));
    sub.h += used;
    sub.hcap -= used;
    const Op16 x1{xh, xl, ldh};
    LATER_CHECK(gemm(sub, 'N', 'T', m, n2, n1, -1.f, x1, l21, 1.f, B + n1 * ldb, ldb));
  }
  return trsm_rlt(b, m, n2, L + n1 + n1 * ldl, ldl, B + n1 * ldb, ldb, xh ? xh + n1 * ldh * 2 : nullptr,
                  xl ? xl + n1 * ldh * 2 : nullptr, ldh, fp32_lim, col >= 0 ? col + n1 : -1);
}

// L X = B, L m x m, B m x n. X's 16-bit copy goes to (xh, ldh) (rows as B).
later_status_t trsm_lln(B3& b, int m, int n, const float* L, int64_t ldl, float* B, int64_t ldb, char* xh, char* xl,
                        int64_t ldh, int fp32_lim = kFp32Trsm) {
  if (m <= NB) {
    const size_t smem = NB * 129 * sizeof(float);
    if (!smem_attr(reinterpret_cast<const void*>(trsm_lln_leaf), smem)) return LATER_ERR_CUDA;
    TraceScope tr(b.st, TRACE_OTHER);
    LATER_CHECK_CUDA(launch_pdl(trsm_lln_leaf, dim3((n + 7) / 8), dim3(256), smem, b.st, m, n, L, ldl, B, ldb, xh, xl,
                                ldh, mode_of(b.o.prec)));
    note_launch();
    return cuda_status(cudaGetLastError());
  }
  const int m1 = half64(m), m2 = m - m1;
  LATER_CHECK(trsm_lln(b, m1, n, L, ldl, B, ldb, xh, xl, ldh, fp32_lim));
  // B2 -= L21 X1   (L21 = L[m1:, :m1], m2 x m1)
  if (m <= fp32_lim) {
    LATER_CHECK(simt_gemm_acc(b.st, m2, m1, n, -1.f, L + m1, ldl, B, ldb, 0, 0, B + m1, ldb));
  } else {
    B3 sub = b;
    Op16 l21;
    size_t used = 0;
    LATER_CHECK(copy16(sub, m2, m1, L + m1, ldl, &l21, &used));
    sub.h += used;
    sub.hcap -= used;
    const Op16 x1{xh, xl, ldh};
    LATER_CHECK(gemm(sub, 'N', 'N', m2, n, m1, -1.f, l21, x1, 1.f, B + m1, ldb));
  }
  return trsm_lln(b, m2, n, L + m1 + m1 * ldl, ldl, B + m1, ldb, xh ? xh + m1 * 2 : nullptr,
                  xl ? xl + m1 * 2 : nullptr, ldh, fp32_lim);
}

// L^T X = B, L m x m lower, B m x n (in place). The update B1 -= L21^T X2 runs
// in FP32 below fp32_lim, else on the tensor cores (16-bit copies converted).
later_status_t trsm_llt(B3& b, int m, int n, const float* L, int64_t ldl, float* B, int64_t ldb,
                        int fp32_lim = kFp32Trsm) {
  if (m <= NB) {
    const size_t smem = NB * 129 * sizeof(float);
    if (!smem_attr(reinterpret_cast<const void*>(trsm_llt_leaf), smem)) return LATER_ERR_CUDA;
    TraceScope tr(b.st, TRACE_OTHER);
    LATER_CHECK_CUDA(launch_pdl(trsm_llt_leaf, dim3((n + 7) / 8), dim3(256), smem, b.st, m, n, L, ldl, B, ldb));
    note_launch();
    return cuda_status(cudaGetLastError());
  }
  const int m1 = half64(m), m2 = m - m1;
  LATER_CHECK(trsm_llt(b, m2, n, L + m1 + m1 * ldl, ldl, B + m1, ldb, fp32_lim));
  // B1 -= L21^T X2   (L21 = L[m1:, :m1], m2 x m1; X2 = B[m1:], m2 x n)
  if (m <= fp32_lim) {
    if (b.ws == nullptr) return LATER_ERR_WORKSPACE;
    LATER_CHECK(simt_tn(b.st, m2, m1, n, L + m1, ldl, B + m1, ldb, B, ldb, 1, *b.ws, -1.f));
  } else {
    B3 sub = b;
    Op16 l21, x2;
    size_t u1 = 0, u2 = 0;
    LATER_CHECK(copy16(sub, m2, m1, L + m1, ldl, &l21, &u1));
    sub.h += u1;
    sub.hcap -= u1;
    LATER_CHECK(copy16(sub, m2, n, B + m1, ldb, &x2, &u2));
    sub.h += u2;
    sub.hcap -= u2;
    LATER_CHECK(gemm(sub, 'T', 'N', m1, n, m2, -1.f, l21, x2, 1.f, B, ldb));
  }
  return trsm_llt(b, m1, n, L, ldl, B, ldb, fp32_lim);
}

// C = L B, L m x m lower, B m x n (its 16-bit copy bh, ldbh), C m x n.
later_status_t trmm_rec(B3& b, int m, int n, const float* L, int64_t ldl, const float* B, int64_t ldb, const Op16& bh,
                        float* C, int64_t ldc) {
  if (m <= NB) {
    const size_t smem = (NB * 129 + NB * 65) * sizeof(float);
    if (!smem_attr(reinterpret_cast<const void*>(trmm_leaf), smem)) return LATER_ERR_CUDA;
    TraceScope tr(b.st, TRACE_OTHER);
    LATER_CHECK_CUDA(launch_pdl(trmm_leaf, dim3((n + 63) / 64), dim3(256), smem, b.st, m, n, L, ldl, B, ldb, C, ldc));
    note_launch();
    return cuda_status(cudaGetLastError());
  }
  const int m1 = half64(m), m2 = m - m1;
  LATER_CHECK(trmm_rec(b, m1, n, L, ldl, B, ldb, bh, C, ldc));
  Op16 bh2{bh.hi ? static_cast<const char*>(bh.hi) + m1 * 2 : nullptr,
           bh.lo ? static_cast<const char*>(bh.lo) + m1 * 2 : nullptr, bh.ld};
  LATER_CHECK(trmm_rec(b, m2, n, L + m1 + m1 * ldl, ldl, B + m1, ldb, bh2, C + m1, ldc));
  // C2 += L21 B1
  if (m <= kFp32Trsm) return simt_gemm_acc(b.st, m2, m1, n, 1.f, L + m1, ldl, B, ldb, 0, 0, C + m1, ldc);
  B3 sub = b;
  Op16 l21;
  size_t used = 0;
  LATER_CHECK(copy16(sub, m2, m1, L + m1, ldl, &l21, &used));
  sub.h += used;
  sub.hcap -= used;
  return gemm(sub, 'N', 'N', m2, n, m1, 1.f, l21, bh, 1.f, C + m1, ldc);
}

// The Cholesky leaves of an n-column block starting at column c (the same
// half64 recursion as potrf_rec); those whose slot is not marked in `done`
// are appended to `out` and marked.
void leaf_blocks(int n, int c, InvBlocks* out, std::vector<char>& done) {
  if (n <= NB) {
    if (!done[c / 64] && out->n < kMaxInvBlocks) {
      out->col[out->n] = c;
      out->w[out->n] = n;
      ++out->n;
      done[c / 64] = 1;
    }
    return;
  }
  const int n1 = half64(n);
  leaf_blocks(n1, c, out, done);
  leaf_blocks(n - n1, c + n1, out, done);
}

// One Cholesky leaf (n <= NB) at factor column `col`; its 32 x 32 diagonal-block inverses go to the table.
// The 256-column nodes of the same recursion over n columns from column c (where the solves split
// 256 columns into two 128-column leaves) whose halves' inverses are in the table; those whose slot
// is not marked in `done2` are appended to `out` and marked.
void pair_blocks(int n, int c, const std::vector<char>& done, InvPairs* out, std::vector<char>& done2) {
  if (n == 2 * NB) {
    if (c % NB == 0 && done[c / 64] && done[c / 64 + 2] && !done2[c / NB] && out->n < kMaxInvPairs) {
      out->col[out->n++] = c;
      done2[c / NB] = 1;
    }
    return;
  }
  if (n < 2 * NB) return;
  const int n1 = half64(n);
  pair_blocks(n1, c, done, out, done2);
  pair_blocks(n - n1, c + n1, done, out, done2);
}

later_status_t potrf_leaf_launch(B3& b, int n, float* A, int64_t lda, int64_t col) {
  const size_t smem = kPotrfLeafSmem;
  if (!smem_attr(reinterpret_cast<const void*>(potrf_leaf), smem)) return LATER_ERR_CUDA;
  TraceScope tr(b.st, TRACE_PANEL);
  float* dinv = b.dinv ? b.dinv + (col / 32) * kDinvSlot : nullptr;
  LATER_CHECK_CUDA(launch_pdl(potrf_leaf, dim3(1), dim3(256), smem, b.st, n, A, lda, device_status_ptr(), dinv));
  note_launch();
  return cuda_status(cudaGetLastError());
}

// Blocked right-looking Cholesky of a block of n <= kFp32Potrf columns (the size the reference hands to
// cuSOLVER's FP32 Spotrf, Cholesky/later_rpotrf.cu:26-35). Per NB-column block k: the leaf factors the
// diagonal block; one solve launch gives X = A[k+1:, k] L_kk^{-T} for all rows below, in place, with its
// hi + lo FP16 pair; one lower-triangle SPLIT3 tensor-core product applies A[k+1:, k+1:] -= X X^T. Three
// launches per block column instead of the recursion's chain of ever smaller solves, updates and
// conversions; every update is FP32-level, as in the recursion.
later_status_t potrf_blocked(B3& b, int n, float* A, int64_t lda, int64_t col) {
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int w = std::min(NB, n - k0);
    float* Akk = A + k0 + static_cast<int64_t>(k0) * lda;
    LATER_CHECK(potrf_leaf_launch(b, w, Akk, lda, col + k0));
    const int r = n - k0 - w;
    if (r == 0) break;
    const int64_t ldx = round_up(r, 8);
    B3 s3 = b;
    s3.o.prec = LATER_PREC_SPLIT3;
    size_t used = 0;
    char* xh = take16(s3, ldx * w, &used);
    if (!xh) return LATER_ERR_WORKSPACE;
    char* xl = xh + ldx * w * 2;
    s3.h += used;
    s3.hcap -= used;
    LATER_CHECK(trsm_rlt(s3, r, w, Akk, lda, Akk + w, lda, xh, xl, ldx, w, col + k0));
    const Op16 x{xh, xl, ldx};
    LATER_CHECK(gemm(s3, 'N', 'T', r, r, w, -1.f, x, x, 1.f, Akk + w + static_cast<int64_t>(w) * lda, lda, nullptr,
                     nullptr, 0, 1));
  }
  return LATER_OK;
}

later_status_t potrf_rec(B3& b, int n, float* A, int64_t lda, int64_t col = 0) {
  if (n <= NB) return potrf_leaf_launch(b, n, A, lda, col);
  if (n <= kFp32Potrf && b.tc_small && b.blocked) return potrf_blocked(b, n, A, lda, col);
  const int n1 = half64(n), n2 = n - n1;
  LATER_CHECK(potrf_rec(b, n1, A, lda, col));
  if (b.leaf_gemm && b.inv_hi && b.inv_done && n2 >= kInvMinRows) {
    // the solve below has n2 rows: invert L11's diagonal blocks that are not inverted yet, all in one launch
    InvBlocks blk{};
    leaf_blocks(n1, static_cast<int>(col), &blk, *b.inv_done);
    if (blk.n > 0) {
      if (!smem_attr(reinterpret_cast<const void*>(trtri_blocks_kernel), kTrtriSmem)) return LATER_ERR_CUDA;
      // A points at the diagonal block starting at column `col`; the kernel takes the factor's origin
      LATER_CHECK_CUDA(launch_pdl(trtri_blocks_kernel, dim3(blk.n), dim3(256), kTrtriSmem, b.st,
                                  static_cast<const float*>(A - col - col * lda), lda, blk, b.inv_hi, b.inv_lo));
      note_launch();
      LATER_CHECK_CUDA(cudaGetLastError());
    }
    if (b.inv2_hi && b.inv2_done) {
      // the solve's 256-column nodes: their inverses from the two halves' (one launch)
      InvPairs prs{};
      pair_blocks(n1, static_cast<int>(col), *b.inv_done, &prs, *b.inv2_done);
      if (prs.n > 0) {
        if (!smem_attr(reinterpret_cast<const void*>(inv256_kernel), kInv256Smem)) return LATER_ERR_CUDA;
        LATER_CHECK_CUDA(launch_pdl(inv256_kernel, dim3(prs.n), dim3(256), kInv256Smem, b.st,
                                    static_cast<const float*>(A - col - col * lda), lda, prs,
                                    static_cast<const __half*>(b.inv_hi), static_cast<const __half*>(b.inv_lo),
                                    b.inv2_hi, b.inv2_lo));
        note_launch();
        LATER_CHECK_CUDA(cudaGetLastError());
      }
    }
  }
  const bool fp32 = n <= kFp32Potrf;
  // A21 <- A21 L11^{-T}; its 16-bit copy is written by the solve. With FP16 (or SPLIT3) operands and
  // the SPLIT3 small updates, the copy is a hi + lo pair (its hi is the FP16 copy), so the SPLIT3 updates
  // of the solve and the syrk below the FP32 thresholds read it instead of converting A21 again.
  const bool pair = b.tc_small && b.o.prec != LATER_PREC_BF16;
  const bool keep = !fp32 || pair;
  const int64_t ldx = round_up(n2, 8);
  size_t used = 0;
  B3 wide = b;
  if (pair) wide.o.prec = LATER_PREC_SPLIT3;  // sizes the pair
  char* xh = keep ? take16(wide, ldx * n1, &used) : nullptr;
  if (keep && !xh) return LATER_ERR_WORKSPACE;
  char* xl = (xh && (pair || b.o.prec == LATER_PREC_SPLIT3)) ? xh + ldx * n1 * 2 : nullptr;
  B3 sub = b;
  sub.h += used;
  sub.hcap -= used;
  LATER_CHECK(trsm_rlt(sub, n2, n1, A, lda, A + n1, lda, xh, xl, ldx, fp32 ? n1 : kFp32Trsm, col));
  // A22 <- A22 - A21 A21^T (lower triangle only)
  if (fp32 && b.tc_small) {
    B3 s3 = sub;
    s3.o.prec = LATER_PREC_SPLIT3;
    Op16 x{xh, xl, ldx};
    if (!xh || !xl) {
      size_t u3 = 0;
      LATER_CHECK(copy16(s3, n2, n1, A + n1, lda, &x, &u3));
      s3.h += u3;
      s3.hcap -= u3;
    }
    LATER_CHECK(gemm(s3, 'N', 'T', n2, n2, n1, -1.f, x, x, 1.f, A + n1 + n1 * lda, lda, nullptr, nullptr, 0, 1));
  } else if (fp32) {
    LATER_CHECK(simt_gemm_acc(b.st, n2, n1, n2, -1.f, A + n1, lda, A + n1, lda, 1, 1, A + n1 + n1 * lda, lda));
  } else {
    const Op16 x{xh, xl, ldx};
    LATER_CHECK(gemm(sub, 'N', 'T', n2, n2, n1, -1.f, x, x, 1.f, A + n1 + n1 * lda, lda, nullptr, nullptr, 0, 1));
  }
  return potrf_rec(b, n2, A + n1 + n1 * lda, lda, col + n1);
}

B3 make_b3(cudaStream_t st, const Options& o, float* work, int64_t lwork, void* hwork, int64_t lhwork) {
  B3 b;
  b.st = st;
  b.o = o;
  b.h = static_cast<char*>(hwork);
  b.hcap = static_cast<size_t>(std::max<int64_t>(lhwork, 0)) * 2;
  if (work && lwork > 4096) {
    b.sc.partial = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(work) + 255) & ~uintptr_t(255));
    b.sc.partial_floats = lwork - 128;
    b.sc.counters = nullptr;
    b.sc.n_counters = 1 << 20;  // split-K needs no counters (separate reduction kernel)
  }
  return b;
}

inline int64_t mult(const Options& o) { return o.prec == LATER_PREC_SPLIT3 ? 2 : 1; }

}  // namespace

// ------------------------------------------------------------ entry points
int64_t rsyrk_hwork(int n, int k, const Options& o) { return (round_up(n, 8) * k + 256) * mult(o); }
int64_t rtrsm_hwork(int m, int n, char leri, const Options& o) {
  // X copy (B-sized) + the largest L21 block
  const int64_t x = round_up(m, 8) * n;
  const int64_t t = (leri == 'r' || leri == 'R') ? static_cast<int64_t>(n) : static_cast<int64_t>(m);
  const int64_t h = t / 2 + 64;
  return (x + round_up(h, 8) * h + 1024) * mult(o);
}
int64_t rtrmm_hwork(int m, int n, const Options& o) {
  const int64_t h = m / 2 + 64;
  return (round_up(m, 8) * n + round_up(h, 8) * h + 1024) * mult(o);
}
int64_t rpotrf_hwork(int n, const Options& o) {
  (void)o;
  // the diagonal blocks' inverses (hi + lo), then the recursion's operand copies in the widest format (SPLIT3)
  const int64_t h = n / 2 + 64;
  const int64_t inv = 2 * inv_slots(n) * kInvSlot + 256;
  const int64_t dinv = dinv_slots(n) * kDinvSlot * 2 + 256;  // FP32 entries, in 16-bit units
  const int64_t inv2 = n > kFp32Potrf ? 2 * inv2_slots(n) * kInv2Slot + 256 : 0;
  return inv + dinv + inv2 +
         (round_up(h, 8) * h + 2 * round_up(h / 2 + 64, 8) * (h / 2 + 64) + round_up(h, 8) * NB + 4096) * 2;
}
int64_t splitk_work() { return static_cast<int64_t>(num_sms()) * 128 * 256 * 2 + 256; }

later_status_t rsyrk(cudaStream_t st, int n, int k, float alpha, const float* A, int64_t lda, float beta, float* C,
                     int64_t ldc, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o) {
  if (o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT3) return LATER_ERR_INVALID_ARG;  // SPLIT2 is rgsqrf's
  if (n < 0 || k < 0 || lda < std::max(n, 1) || ldc < std::max(n, 1) || !A || !C) return LATER_ERR_INVALID_ARG;
  if (n == 0) return LATER_OK;
  if (!hwork || lhwork < rsyrk_hwork(n, k, o) || (reinterpret_cast<uintptr_t>(hwork) & 15)) return LATER_ERR_WORKSPACE;
  B3 b = make_b3(st, o, work, lwork, hwork, lhwork);
  if (k == 0) return axpy2d(st, n, n, beta - 1.f, C, ldc, C, ldc);  // C = beta C (lower and upper alike)
  Op16 a;
  size_t used = 0;
  LATER_CHECK(copy16(b, n, k, A, lda, &a, &used));
  return gemm(b, 'N', 'T', n, n, k, alpha, a, a, beta, C, ldc, nullptr, nullptr, 0, 1);
}

later_status_t rtrsm(cudaStream_t st, char uplo, char leri, char trans, int m, int n, const float* A, int64_t lda,
                     float* B, int64_t ldb, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                     const Options& o) {
  return rtrsm_lim(st, uplo, leri, trans, m, n, A, lda, B, ldb, work, lwork, hwork, lhwork, o, kFp32Trsm);
}

later_status_t rtrsm_lim(cudaStream_t st, char uplo, char leri, char trans, int m, int n, const float* A,
                         int64_t lda, float* B, int64_t ldb, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                         const Options& o, int fp32_lim) {
  if (o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT3) return LATER_ERR_INVALID_ARG;  // SPLIT2 is rgsqrf's
  auto lc = [](char c) { return static_cast<char>(c | 0x20); };
  const char u = lc(uplo), s = lc(leri), t = lc(trans);
  const bool lln = (u == 'l' && s == 'l' && t == 'n');
  const bool lrt = (u == 'l' && s == 'r' && t == 't');
  const bool llt = (u == 'l' && s == 'l' && t == 't');  // extension: L^T X = B
  if (!lln && !lrt && !llt) return LATER_ERR_NOT_SUPPORTED;
  if (m < 0 || n < 0 || !A || !B || ldb < std::max(m, 1) || lda < std::max(lrt ? n : m, 1)) return LATER_ERR_INVALID_ARG;
  if (m == 0 || n == 0) return LATER_OK;
  if (!hwork || lhwork < rtrsm_hwork(m, n, s, o) || (reinterpret_cast<uintptr_t>(hwork) & 15))
    return LATER_ERR_WORKSPACE;
  B3 b = make_b3(st, o, work, lwork, hwork, lhwork);
  if (llt) {
    Arena ws(work, work ? static_cast<size_t>(std::max<int64_t>(lwork, 0)) * sizeof(float) : 0);
    b.ws = work ? &ws : nullptr;
    return trsm_llt(b, m, n, A, lda, B, ldb, fp32_lim);
  }
  const int64_t ldx = round_up(m, 8);
  size_t used = 0;
  char* xh = take16(b, ldx * n, &used);
  if (!xh) return LATER_ERR_WORKSPACE;
  char* xl = o.prec == LATER_PREC_SPLIT3 ? xh + ldx * n * 2 : nullptr;
  b.h += used;
  b.hcap -= used;
  return lln ? trsm_lln(b, m, n, A, lda, B, ldb, xh, xl, ldx, fp32_lim)
             : trsm_rlt(b, m, n, A, lda, B, ldb, xh, xl, ldx, fp32_lim);
}

later_status_t rtrmm(cudaStream_t st, int m, int n, const float* A, int64_t lda, const float* B, int64_t ldb,
                     float* C, int64_t ldc, float* work, int64_t lwork, void* hwork, int64_t lhwork,
                     const Options& o) {
  if (o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT3) return LATER_ERR_INVALID_ARG;  // SPLIT2 is rgsqrf's
  if (m < 0 || n < 0 || !A || !B || !C || lda < std::max(m, 1) || ldb < std::max(m, 1) || ldc < std::max(m, 1))
    return LATER_ERR_INVALID_ARG;
  if (m == 0 || n == 0) return LATER_OK;
  if (!hwork || lhwork < rtrmm_hwork(m, n, o) || (reinterpret_cast<uintptr_t>(hwork) & 15)) return LATER_ERR_WORKSPACE;
  B3 b = make_b3(st, o, work, lwork, hwork, lhwork);
  Op16 bh;
  size_t used = 0;
  LATER_CHECK(copy16(b, m, n, B, ldb, &bh, &used));
  b.h += used;
  b.hcap -= used;
  return trmm_rec(b, m, n, A, lda, B, ldb, bh, C, ldc);
}

later_status_t rpotrf(cudaStream_t st, char uplo, int n, float* A, int64_t lda, float* work, int64_t lwork,
                      void* hwork, int64_t lhwork, const Options& o) {
  if (o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT3) return LATER_ERR_INVALID_ARG;  // SPLIT2 is rgsqrf's
  if ((uplo | 0x20) != 'l') return LATER_ERR_NOT_SUPPORTED;
  if (n < 0 || !A || lda < std::max(n, 1)) return LATER_ERR_INVALID_ARG;
  if (n == 0) return LATER_OK;
  if (n > NB && (!hwork || lhwork < rpotrf_hwork(n, o) || (reinterpret_cast<uintptr_t>(hwork) & 15)))
    return LATER_ERR_WORKSPACE;
  B3 b = make_b3(st, o, work, lwork, hwork, lhwork);
  if (n > NB) {
    // inverses of the factor's diagonal blocks first in hwork; the recursion's scratch after them
    b.tc_small = true;
    b.blocked = potrf_blocked_enabled();
    b.leaf_gemm = o.prec != LATER_PREC_SPLIT3;  // SPLIT3 keeps FP32 substitution in the block solves
    const int64_t slots = inv_slots(n) * kInvSlot;
    if (b.leaf_gemm) {
      b.inv_hi = static_cast<__half*>(hwork);
      b.inv_lo = b.inv_hi + slots;
    }
    size_t skip = static_cast<size_t>(2 * slots) * 2;
    // then the FP32 table of the 32 x 32 diagonal-block inverses (256-byte aligned)
    const uintptr_t d = (reinterpret_cast<uintptr_t>(b.h) + skip + 255) & ~uintptr_t(255);
    b.dinv = reinterpret_cast<float*>(d);
    skip = (d - reinterpret_cast<uintptr_t>(b.h)) + static_cast<size_t>(dinv_slots(n)) * kDinvSlot * sizeof(float);
    if (b.leaf_gemm && n > kFp32Potrf && inv2_enabled()) {
      // then the 256-column inverses (256-byte aligned)
      const uintptr_t w = (reinterpret_cast<uintptr_t>(b.h) + skip + 255) & ~uintptr_t(255);
      b.inv2_hi = reinterpret_cast<__half*>(w);
      b.inv2_lo = b.inv2_hi + inv2_slots(n) * kInv2Slot;
      skip = (w - reinterpret_cast<uintptr_t>(b.h)) + static_cast<size_t>(2 * inv2_slots(n) * kInv2Slot) * 2;
    }
    b.h += skip;
    b.hcap = b.hcap > skip ? b.hcap - skip : 0;
  }
  std::vector<char> done(static_cast<size_t>(inv_slots(std::max(n, 1))), 0);
  std::vector<char> done2(static_cast<size_t>(inv2_slots(std::max(n, 1))), 0);
  b.inv_done = &done;
  b.inv2_done = &done2;
  return potrf_rec(b, n, A, lda);
}

}  // namespace later

// Tall-skinny FP32 panel kernels for the rgsqrf leaf.
//
// The reference factors each 32-column sub-panel with a TSQR tree of
// mgs_kernel2 launches (QR/panel.cu:65-134, 246-325): MGS of every 256-row
// block, the 32x32 R factors stacked and factored again until one block is
// left, then each block's Q multiplied by its slice of the stacked Q with
// cublasSgemmStridedBatched. The 128-wide leaf glues four such panels with six
// FP32 cublasSgemm block-CGS updates (QR/panel.cu:10-63).
//
// Here the whole reduction tree is one launch (tsqr_reduce_kernel): every CTA
// factors its 256 x 32 block with MGS held in registers (warp = column,
// 8 rows per lane), writes Q in place and its R into the next level's stack,
// then takes an atomic ticket; the last CTA of each group of eight carries on
// with the next level, so no CTA ever waits on another. A second launch
// (tsqr_apply_kernel) composes each block's path through the tree (32x32
// products) and writes the final Q in FP32 together with its 16-bit copy, so
// the tensor-core GEMMs that follow need no conversion pass.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "panel.cuh"
#include "runtime.cuh"

namespace later {

namespace {

constexpr int PB = 32;    // panel width
constexpr int BR = 256;   // rows per TSQR block
constexpr int RPL = BR / 32;  // rows per lane

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// MGS of one (<=256) x 32 block held in registers. Warp w owns column w; lane
// l holds rows l + 32 t. q buffers are double-buffered so each step needs one
// barrier. Columns beyond the block's row count are exactly dependent and are
// set to zero (R row zero) instead of normalising round-off.
__device__ void mgs_block(float (&a)[RPL], int mm, float* qbuf /*2*BR*/, float* Rs /*32x33*/) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll 1
  for (int k = 0; k < PB; ++k) {
    float* q = qbuf + (k & 1) * BR;
    if (w == k) {
      float s = 0.f;
#pragma unroll
      for (int t = 0; t < RPL; ++t) s += a[t] * a[t];
      s = warp_sum(s);
      float nrm = sqrtf(s);
      if (k >= mm || !(nrm > 0.f)) nrm = 0.f;
      const float inv = nrm > 0.f ? 1.f / nrm : 0.f;
#pragma unroll
      for (int t = 0; t < RPL; ++t) {
        a[t] *= inv;
        q[l + 32 * t] = a[t];
      }
      if (l == 0) Rs[k * 33 + k] = nrm;
    }
    __syncthreads();
    if (w > k) {
      float d = 0.f;
#pragma unroll
      for (int t = 0; t < RPL; ++t) d += q[l + 32 * t] * a[t];
      d = warp_sum(d);
#pragma unroll
      for (int t = 0; t < RPL; ++t) a[t] -= d * q[l + 32 * t];
      if (l == 0) Rs[k * 33 + w] = d;  // Rs[row k][col w]
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(1024, 1) tsqr_reduce_kernel(TsqrPlan P) {
  __shared__ float qbuf[2 * BR];
  __shared__ float Rs[PB * 33];
  __shared__ int last;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  int L = 0;
  int b = blockIdx.x;
  while (true) {
    float* X = P.lev[L];
    const int64_t ld = P.ld[L];
    const int rows = P.rows[L];
    const int r0 = b * BR;
    const int mm = min(BR, rows - r0);
    float a[RPL];
#pragma unroll
    for (int t = 0; t < RPL; ++t) {
      const int r = l + 32 * t;
      a[t] = (r < mm) ? __ldcg(&X[r0 + r + static_cast<int64_t>(w) * ld]) : 0.f;
    }
    mgs_block(a, mm, qbuf, Rs);
    // Q in place.
#pragma unroll
    for (int t = 0; t < RPL; ++t) {
      const int r = l + 32 * t;
      if (r < mm) X[r0 + r + static_cast<int64_t>(w) * ld] = a[t];
    }
    // R: to the output at the root, else into the next level's stack.
    const bool root = (P.nblk[L] == 1);
    float* Ro = root ? P.R : P.lev[L + 1] + 32 * b;
    const int64_t ldo = root ? P.ldr : P.ld[L + 1];
    {
      const int i = l, j = w;  // element (i, j) of the 32x32 R
      Ro[i + static_cast<int64_t>(j) * ldo] = (i <= j) ? Rs[i * 33 + j] : 0.f;
    }
    if (root) break;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      const int g = b >> 3;
      const int gsize = min(8, P.nblk[L] - 8 * g);
      int* c = P.counters + P.cnt_off[L] + g;
      const int prev = atomicAdd(c, 1);
      last = (prev == gsize - 1);
      if (last) *c = 0;
    }
    __syncthreads();
    if (!last) break;
    __threadfence();
    b >>= 3;
    ++L;
  }
}

// Each CTA finishes 256 rows of Q: T = product of its 32x32 path slices
// through the tree, Q = Q0 * T, written in FP32 and as the 16-bit copy.
__global__ void __launch_bounds__(256) tsqr_apply_kernel(TsqrPlan P, void* qh, void* ql, int64_t ldh,
                                                         int out_mode) {
  __shared__ float T[PB * 33];
  __shared__ float U[PB * 33];
  const int b = blockIdx.x;
  const int tid = threadIdx.x;
  const int top = P.nlev - 1;
  // T = slice of the top level, then T = slice_L * T down to level 1.
  if (top == 0) {
    for (int e = tid; e < PB * PB; e += 256) T[(e % PB) * 33 + e / PB] = (e % PB == e / PB) ? 1.f : 0.f;
  } else {
    const int bt = b >> (3 * (top - 1));  // block index at level top-1
    for (int e = tid; e < PB * PB; e += 256) {
      const int i = e % PB, j = e / PB;
      T[i * 33 + j] = __ldcg(&P.lev[top][32 * bt + i + static_cast<int64_t>(j) * P.ld[top]]);
    }
    for (int L = top - 1; L >= 1; --L) {
      __syncthreads();
      const int bl = b >> (3 * (L - 1));
      for (int e = tid; e < PB * PB; e += 256) {
        const int i = e % PB, j = e / PB;
        float s = 0.f;
#pragma unroll 8
        for (int k = 0; k < PB; ++k)
          s += __ldcg(&P.lev[L][32 * bl + i + static_cast<int64_t>(k) * P.ld[L]]) * T[k * 33 + j];
        U[i * 33 + j] = s;
      }
      __syncthreads();
      for (int e = tid; e < PB * PB; e += 256) T[(e % PB) * 33 + e / PB] = U[(e % PB) * 33 + e / PB];
    }
  }
  __syncthreads();
  const int row = b * BR + tid;
  if (row >= P.rows[0]) return;
  float* X = P.lev[0];
  const int64_t ld = P.ld[0];
  float q[PB];
#pragma unroll
  for (int k = 0; k < PB; ++k) q[k] = __ldcg(&X[row + static_cast<int64_t>(k) * ld]);
#pragma unroll 4
  for (int j = 0; j < PB; ++j) {
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < PB; ++k) s += q[k] * T[k * 33 + j];
    X[row + static_cast<int64_t>(j) * ld] = s;
    if (qh) {
      const int64_t o = row + static_cast<int64_t>(j) * ldh;
      if (out_mode == 1) {
        reinterpret_cast<__nv_bfloat16*>(qh)[o] = __float2bfloat16_rn(s);
      } else {
        const __half h = __float2half_rn(s);
        reinterpret_cast<__half*>(qh)[o] = h;
        if (out_mode == 2) reinterpret_cast<__half*>(ql)[o] = __float2half_rn((s - __half2float(h)) * 2048.f);
      }
    }
  }
}

// ---------------------------------------------------------- FP32 SIMT GEMMs
// Partial products P[c] = X[rows of chunk c]^T Y[rows of chunk c] for k1, k2 <= 64.
constexpr int CH = 64;  // rows per shared-memory tile; a CTA covers `rpc` rows (multiple of CH)
__global__ void __launch_bounds__(256) tn_partial_kernel(int m, int rpc, int k1, int k2, const float* __restrict__ X,
                                                         int64_t ldx, const float* __restrict__ Y, int64_t ldy,
                                                         float* __restrict__ part) {
  __shared__ float Xs[CH][65];
  __shared__ float Ys[CH][65];
  const int c = blockIdx.x;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int r0 = c * rpc; r0 < min(m, (c + 1) * rpc); r0 += CH) {
    const int mm = min(CH, m - r0);
    __syncthreads();
    for (int e = threadIdx.x; e < CH * 64; e += 256) {
      const int r = e % CH, j = e / CH;
      Xs[r][j] = (r < mm && j < k1) ? __ldcg(&X[r0 + r + static_cast<int64_t>(j) * ldx]) : 0.f;
      Ys[r][j] = (r < mm && j < k2) ? __ldcg(&Y[r0 + r + static_cast<int64_t>(j) * ldy]) : 0.f;
    }
    __syncthreads();
#pragma unroll 4
    for (int r = 0; r < CH; ++r) {
      float x[4], y[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        x[u] = Xs[r][tx + 16 * u];
        y[u] = Ys[r][ty + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] += x[u] * y[v];
    }
  }
  float* out = part + static_cast<int64_t>(c) * 64 * 64;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) out[(tx + 16 * u) + 64 * (ty + 16 * v)] = acc[u][v];
}

// R[i,j] (+)= sum over chunks in order (deterministic).
__global__ void tn_reduce_kernel(int nch, int k1, int k2, const float* __restrict__ part, float* R, int64_t ldr,
                                 int accumulate) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 64 * 64) return;
  const int i = e % 64, j = e / 64;
  if (i >= k1 || j >= k2) return;
  float s = 0.f;
  for (int c = 0; c < nch; ++c) s += __ldcg(&part[static_cast<int64_t>(c) * 4096 + e]);
  float* o = &R[i + static_cast<int64_t>(j) * ldr];
  *o = accumulate ? *o + s : s;
}

// Y[rows] -= X[rows] * S  with S (k1 x k2, k <= 64) from R (ldr).
__global__ void __launch_bounds__(256) nn_update_kernel(int m, int k1, int k2, const float* __restrict__ X,
                                                        int64_t ldx, const float* __restrict__ S, int64_t lds,
                                                        float* Y, int64_t ldy) {
  __shared__ float Ss[64][65];
  for (int e = threadIdx.x; e < 64 * 64; e += 256) {
    const int i = e % 64, j = e / 64;
    Ss[i][j] = (i < k1 && j < k2) ? S[i + static_cast<int64_t>(j) * lds] : 0.f;
  }
  __syncthreads();
  const int r = blockIdx.x * 128 + (threadIdx.x & 127);
  const int half = threadIdx.x >> 7;  // columns [32 half, 32 half + 32)
  if (r >= m) return;
  float x[64];
#pragma unroll
  for (int k = 0; k < 64; ++k) x[k] = (k < k1) ? __ldcg(&X[r + static_cast<int64_t>(k) * ldx]) : 0.f;
#pragma unroll 2
  for (int jj = 0; jj < 32; ++jj) {
    const int j = 32 * half + jj;
    if (j >= k2) break;
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 64; ++k) s += x[k] * Ss[k][j];
    float* y = &Y[r + static_cast<int64_t>(j) * ldy];
    *y -= s;
  }
}

}  // namespace

// Level sizes of the TSQR tree for an m-row panel; returns the workspace need.
void tsqr_plan_sizes(int m, int* nlev, int rows[kMaxTsqrLevels], int nblk[kMaxTsqrLevels], int64_t* stack_floats,
                     int* ncounters) {
  int L = 0;
  int r = m;
  int64_t st = 0;
  int cnt = 0;
  while (true) {
    rows[L] = r;
    nblk[L] = (r + BR - 1) / BR;
    if (nblk[L] == 1 || L == kMaxTsqrLevels - 1) break;
    cnt += (nblk[L] + 7) / 8;
    r = 32 * nblk[L];
    st += round_up(r, 64) * 32;
    ++L;
  }
  *nlev = L + 1;
  *stack_floats = st;
  *ncounters = cnt;
}

later_status_t tsqr_panel(cudaStream_t s, int m, float* A, int64_t lda, float* R, int64_t ldr, void* qh, void* ql,
                          int64_t ldh, int out_prec, Arena& ws, int* counters_zeroed) {
  TsqrPlan P{};
  int64_t stack = 0;
  int ncnt = 0;
  tsqr_plan_sizes(m, &P.nlev, P.rows, P.nblk, &stack, &ncnt);
  if (P.nblk[P.nlev - 1] != 1 || ncnt > 2048) return LATER_ERR_NOT_SUPPORTED;  // m beyond the tree capacity
  P.lev[0] = A;
  P.ld[0] = lda;
  const size_t mark = ws.used();
  for (int L = 1; L < P.nlev; ++L) {
    P.ld[L] = round_up(P.rows[L], 64);
    P.lev[L] = ws.take<float>(P.ld[L] * 32);
    if (!P.lev[L]) return LATER_ERR_WORKSPACE;
  }
  int off = 0;
  for (int L = 0; L < P.nlev - 1; ++L) {
    P.cnt_off[L] = off;
    off += (P.nblk[L] + 7) / 8;
  }
  P.counters = counters_zeroed;
  P.R = R;
  P.ldr = ldr;
  if (ws.sizing()) {
    ws.reset(mark);
    return LATER_OK;
  }
  tsqr_reduce_kernel<<<P.nblk[0], 1024, 0, s>>>(P);
  LATER_CHECK_CUDA(cudaGetLastError());
  const int mode = out_prec == LATER_PREC_BF16 ? 1 : (out_prec == LATER_PREC_SPLIT3 ? 2 : 0);
  tsqr_apply_kernel<<<P.nblk[0], 256, 0, s>>>(P, qh, ql, ldh, mode);
  LATER_CHECK_CUDA(cudaGetLastError());
  ws.reset(mark);
  return LATER_OK;
}

later_status_t simt_tn(cudaStream_t s, int m, int k1, int k2, const float* X, int64_t ldx, const float* Y,
                       int64_t ldy, float* R, int64_t ldr, int accumulate, Arena& ws) {
  // One partial 64x64 tile per CTA; as many CTAs (up to one per 128 rows) as
  // the workspace holds partial tiles for.
  int nch = (m + 127) / 128;
  const int64_t fit = static_cast<int64_t>(ws.remaining() / sizeof(float)) / 4096 - 1;
  if (!ws.sizing() && fit < nch) nch = fit < 1 ? 1 : static_cast<int>(fit);
  const int rpc = static_cast<int>(round_up((m + nch - 1) / nch, CH));
  nch = (m + rpc - 1) / rpc;
  const size_t mark = ws.used();
  float* part = ws.take<float>(static_cast<size_t>(nch) * 4096);
  if (!part) return LATER_ERR_WORKSPACE;
  if (ws.sizing()) {
    ws.reset(mark);
    return LATER_OK;
  }
  tn_partial_kernel<<<nch, 256, 0, s>>>(m, rpc, k1, k2, X, ldx, Y, ldy, part);
  LATER_CHECK_CUDA(cudaGetLastError());
  tn_reduce_kernel<<<16, 256, 0, s>>>(nch, k1, k2, part, R, ldr, accumulate);
  LATER_CHECK_CUDA(cudaGetLastError());
  ws.reset(mark);
  return LATER_OK;
}

later_status_t simt_nn_sub(cudaStream_t s, int m, int k1, int k2, const float* X, int64_t ldx, const float* S,
                           int64_t lds, float* Y, int64_t ldy) {
  nn_update_kernel<<<(m + 127) / 128, 256, 0, s>>>(m, k1, k2, X, ldx, S, lds, Y, ldy);
  return cuda_status(cudaGetLastError());
}

}  // namespace later

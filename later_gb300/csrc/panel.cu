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
// factors its 256-row block with block MGS held in registers (4 columns per warp),
// writes Q in place and its R into the next level's stack, then takes an
// atomic ticket; the last CTA of each group of eight carries on with the next
// level, so no CTA ever waits on another CTA. A second launch
// (tsqr_apply_kernel) composes each block's path through the tree (32x32
// products) and writes the final Q in FP32 together with its 16-bit copy, so
// the tensor-core GEMMs that follow need no conversion pass.
#include <algorithm>

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "panel.cuh"
#include "ptx.cuh"
#include "runtime.cuh"
#include "tsqr_dev.cuh"

namespace later {

namespace {

constexpr int APPLY_ROWS = 128;

__global__ void __launch_bounds__(256) tsqr_reduce_kernel(TsqrPlan P) {
  __shared__ TsqrReduceSmem sm;
  tsqr_reduce_block(P, blockIdx.x, sm);
}

__global__ void __launch_bounds__(APPLY_ROWS) tsqr_apply_kernel(TsqrPlan P, void* qh, void* ql, int64_t ldh,
                                                                int out_mode) {
  __shared__ TsqrApplySmem sm;
  tsqr_apply_rows(P, blockIdx.x * APPLY_ROWS, qh, ql, ldh, out_mode, sm);
}

// ---------------------------------------------------------- FP32 SIMT GEMMs
// Partial products P[c][t] = X[rows of chunk c]^T Y[rows of chunk c] for the
// 64x64 output tile t = (ti, tj): grid (chunks, tiles_i * tiles_j).
constexpr int CH = 64;  // rows per shared-memory tile; a CTA covers `rpc` rows (multiple of CH)
__global__ void __launch_bounds__(256) tn_partial_kernel(int m, int rpc, int k1, int k2, const float* __restrict__ X,
                                                         int64_t ldx, const float* __restrict__ Y, int64_t ldy,
                                                         float* __restrict__ part) {
  __shared__ float Xs[CH][65];
  __shared__ float Ys[CH][65];
  const int c = blockIdx.x;
  const int ti_n = (k1 + 63) / 64;
  const int ti = blockIdx.y % ti_n, tj = blockIdx.y / ti_n;
  const int i0 = ti * 64, j0 = tj * 64;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int r0 = c * rpc; r0 < min(m, (c + 1) * rpc); r0 += CH) {
    const int mm = min(CH, m - r0);
    __syncthreads();
    float xv[CH * 64 / 256], yv[CH * 64 / 256];
#pragma unroll
    for (int u = 0; u < CH * 64 / 256; ++u) {
      const int e = threadIdx.x + 256 * u;
      const int r = e % CH, j = e / CH;
      const bool in = r < mm;
      xv[u] = (in && i0 + j < k1) ? __ldcg(&X[r0 + r + static_cast<int64_t>(i0 + j) * ldx]) : 0.f;
      yv[u] = (in && j0 + j < k2) ? __ldcg(&Y[r0 + r + static_cast<int64_t>(j0 + j) * ldy]) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < CH * 64 / 256; ++u) {
      const int e = threadIdx.x + 256 * u;
      Xs[e % CH][e / CH] = xv[u];
      Ys[e % CH][e / CH] = yv[u];
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
  float* out = part + (static_cast<int64_t>(c) * gridDim.y + blockIdx.y) * 4096;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) out[(tx + 16 * u) + 64 * (ty + 16 * v)] = acc[u][v];
}

// R[i,j] (+)= sum over chunks, deterministic: 32 outputs x 8 slices per block;
// slice j sums chunks j, j+8, ... in order, slices combined in a fixed tree.
__global__ void __launch_bounds__(256) tn_reduce_kernel(int nch, int ntiles, int k1, int k2,
                                                        const float* __restrict__ part, float* R, int64_t ldr,
                                                        int accumulate, float alpha) {
  __shared__ float sl[8][33];
  const int t = blockIdx.x / 128;                     // output tile
  const int e = (blockIdx.x % 128) * 32 + threadIdx.x % 32;  // element of the 64x64 tile
  const int j = threadIdx.x / 32;
  float acc = 0.f;
#pragma unroll 8
  for (int c = j; c < nch; c += 8) acc += __ldcg(&part[(static_cast<int64_t>(c) * ntiles + t) * 4096 + e]);
  sl[j][threadIdx.x % 32] = acc;
  __syncthreads();
  if (j != 0) return;
  const int l = threadIdx.x;
  const float s = ((sl[0][l] + sl[1][l]) + (sl[2][l] + sl[3][l])) + ((sl[4][l] + sl[5][l]) + (sl[6][l] + sl[7][l]));
  const int ti_n = (k1 + 63) / 64;
  const int i = (t % ti_n) * 64 + e % 64, jj = (t / ti_n) * 64 + e / 64;
  if (i >= k1 || jj >= k2) return;
  float* o = &R[i + static_cast<int64_t>(jj) * ldr];
  *o = accumulate ? *o + alpha * s : alpha * s;
}

// Y[rows, cols] += alpha X[rows, :] S[:, cols] with S (k1 x k2; stored
// transposed when s_trans). One CTA per 64 rows x 64 columns; the inner
// dimension is walked in chunks of 64 with X and alpha*S staged k-major in
// shared memory; each thread accumulates 4 consecutive rows x 4 consecutive
// columns from float4 reads, and adds the sum into Y once at the end.
// Optional 16-bit copy of the updated Y (mode 0 fp16, 1 bf16, 2 split3 hi/lo).
constexpr int NNR = 64;
__global__ void __launch_bounds__(256) nn_update_kernel(int m, int k1, int k2, float alpha, const float* __restrict__ X,
                                                        int64_t ldx, const float* __restrict__ S, int64_t lds,
                                                        int s_trans, int lower, float* __restrict__ Y, int64_t ldy,
                                                        void* yh, void* yl, int64_t ldh, int mode) {
  __shared__ __align__(16) float Ss[64][68];  // [k][col]
  __shared__ __align__(16) float Xs[64][68];  // [k][row]
  const int r0 = blockIdx.x * NNR;
  const int c0 = blockIdx.y * 64;
  if (lower && r0 + NNR - 1 < c0) return;  // tile entirely above the diagonal
  const int mm = min(NNR, m - r0);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // rows 4 tx + u, cols 4 ty + v
  float acc[4][4] = {};
  for (int k0 = 0; k0 < k1; k0 += 64) {
    float sv[16], xv[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = threadIdx.x + 256 * u;
      const int lo = e % 64, hi = e / 64;
      xv[u] = (lo < mm && k0 + hi < k1) ? __ldcg(&X[r0 + lo + static_cast<int64_t>(k0 + hi) * ldx]) : 0.f;
      if (s_trans)  // S[c][k] at c + k lds: lo = column, hi = k
        sv[u] = (c0 + lo < k2 && k0 + hi < k1) ? S[c0 + lo + static_cast<int64_t>(k0 + hi) * lds] : 0.f;
      else          // S[k][c] at k + c lds: lo = k, hi = column
        sv[u] = (k0 + lo < k1 && c0 + hi < k2) ? S[k0 + lo + static_cast<int64_t>(c0 + hi) * lds] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = threadIdx.x + 256 * u;
      const int lo = e % 64, hi = e / 64;
      Xs[hi][lo] = xv[u];
      if (s_trans)
        Ss[hi][lo] = alpha * sv[u];
      else
        Ss[lo][hi] = alpha * sv[u];
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < 64; ++k) {
      const float4 xr = *reinterpret_cast<const float4*>(&Xs[k][4 * tx]);
      const float4 sr = *reinterpret_cast<const float4*>(&Ss[k][4 * ty]);
      const float xa[4] = {xr.x, xr.y, xr.z, xr.w};
      const float sa[4] = {sr.x, sr.y, sr.z, sr.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] += xa[u] * sa[v];
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int i = 4 * tx + u, j = c0 + 4 * ty + v;
      if (i < mm && j < k2 && (!lower || r0 + i >= j)) {
        float* yp = &Y[r0 + i + static_cast<int64_t>(j) * ldy];
        const float val = *yp + acc[u][v];
        *yp = val;
        if (yh) {
          const int64_t o = r0 + i + static_cast<int64_t>(j) * ldh;
          if (mode == 1) {
            reinterpret_cast<__nv_bfloat16*>(yh)[o] = __float2bfloat16_rn(val);
          } else {
            const __half h = __float2half_rn(val);
            reinterpret_cast<__half*>(yh)[o] = h;
            if (mode == 2) reinterpret_cast<__half*>(yl)[o] = __float2half_rn((val - __half2float(h)) * 2048.f);
          }
        }
      }
    }
}

}  // namespace

// Level sizes of the TSQR tree for an m-row panel: 256-row blocks at every
// level, eight 32x32 R factors stacked per block of the next level (the
// reference's tree shape, QR/panel.cu:87-133). A 16384-row panel has three
// levels (64, 8, 1 blocks).
void tsqr_plan_sizes(int m, TsqrPlan* P, int64_t* stack_floats, int* ncounters) {
  int L = 0;
  int r = m;
  int64_t st = 0;
  int cnt = 0;
  P->div[0] = 1;
  while (true) {
    P->br[L] = BR;
    P->rows[L] = r;
    P->nblk[L] = (r + BR - 1) / BR;
    if (P->nblk[L] == 1 || L == kMaxTsqrLevels - 1) break;
    P->cnt_off[L] = cnt;
    cnt += (P->nblk[L] + kGroup - 1) / kGroup;
    r = PB * P->nblk[L];
    P->div[L + 1] = P->div[L] * kGroup;
    st += round_up(r, 64) * PB;
    ++L;
  }
  P->maxbr = BR;
  P->nlev = L + 1;
  *stack_floats = st;
  *ncounters = cnt;
}

later_status_t tsqr_panel(cudaStream_t s, int m, float* A, int64_t lda, float* R, int64_t ldr, void* qh, void* ql,
                          int64_t ldh, int out_prec, Arena& ws, int* counters_zeroed, long long budget, int ncols) {
  if (ncols < 1 || ncols > PB) return LATER_ERR_INVALID_ARG;
  TsqrPlan P{};
  P.ncols = ncols;
  int64_t stack = 0;
  int ncnt = 0;
  tsqr_plan_sizes(m, &P, &stack, &ncnt);
  if (P.nblk[P.nlev - 1] != 1 || ncnt > 2048) return LATER_ERR_NOT_SUPPORTED;  // m beyond the tree capacity
  P.lev[0] = A;
  P.ld[0] = lda;
  const size_t mark = ws.used();
  for (int L = 1; L < P.nlev; ++L) {
    P.ld[L] = round_up(P.rows[L], 64);
    P.lev[L] = ws.take<float>(P.ld[L] * 32);
    if (!P.lev[L]) return LATER_ERR_WORKSPACE;
  }
  P.counters = counters_zeroed;
  P.R = R;
  P.ldr = ldr;
  P.status = device_status_ptr();
  P.budget = budget > 0 ? budget : kDefaultBudgetCycles;
  if (ws.sizing()) {
    ws.reset(mark);
    return LATER_OK;
  }
  TraceScope trace(s, TRACE_PANEL);
  tsqr_reduce_kernel<<<P.nblk[0], 256, 0, s>>>(P);
  note_launch();
  LATER_CHECK_CUDA(cudaGetLastError());
  const int mode = out_prec == LATER_PREC_BF16 ? 1 : (out_prec == LATER_PREC_SPLIT3 ? 2 : 0);
  tsqr_apply_kernel<<<(m + APPLY_ROWS - 1) / APPLY_ROWS, APPLY_ROWS, 0, s>>>(P, qh, ql, ldh, mode);
  note_launch();
  LATER_CHECK_CUDA(cudaGetLastError());
  ws.reset(mark);
  return LATER_OK;
}

later_status_t simt_tn(cudaStream_t s, int m, int k1, int k2, const float* X, int64_t ldx, const float* Y,
                       int64_t ldy, float* R, int64_t ldr, int accumulate, Arena& ws, float alpha) {
  if (m <= 0 || k1 <= 0 || k2 <= 0) return LATER_OK;
  // Partial 64x64 tiles per (row chunk, output tile); as many row chunks (up
  // to one per 128 rows, at most 256) as the workspace holds.
  const int ntiles = ((k1 + 63) / 64) * ((k2 + 63) / 64);
  int nch = (m + 127) / 128;
  if (nch > 256) nch = 256;
  if (nch * ntiles > 4096) nch = std::max(1, 4096 / ntiles);
  const int64_t fit = static_cast<int64_t>(ws.remaining() / sizeof(float)) / (4096LL * ntiles) - 1;
  if (!ws.sizing() && fit < nch) nch = fit < 1 ? 1 : static_cast<int>(fit);
  const int rpc = static_cast<int>(round_up((m + nch - 1) / nch, CH));
  nch = (m + rpc - 1) / rpc;
  const size_t mark = ws.used();
  float* part = ws.take<float>(static_cast<size_t>(nch) * ntiles * 4096);
  if (!part) return LATER_ERR_WORKSPACE;
  if (ws.sizing()) {
    ws.reset(mark);
    return LATER_OK;
  }
  TraceScope trace(s, TRACE_LEAF_GEMM, 2.0 * m * k1 * k2);
  tn_partial_kernel<<<dim3(nch, ntiles), 256, 0, s>>>(m, rpc, k1, k2, X, ldx, Y, ldy, part);
  note_launch();
  LATER_CHECK_CUDA(cudaGetLastError());
  tn_reduce_kernel<<<ntiles * 128, 256, 0, s>>>(nch, ntiles, k1, k2, part, R, ldr, accumulate, alpha);
  note_launch();
  LATER_CHECK_CUDA(cudaGetLastError());
  ws.reset(mark);
  return LATER_OK;
}

later_status_t simt_gemm_acc(cudaStream_t s, int m, int k1, int k2, float alpha, const float* X, int64_t ldx,
                             const float* S, int64_t lds, int s_trans, int lower, float* Y, int64_t ldy, void* yh,
                             void* yl, int64_t ldh, int out_prec) {
  if (m <= 0 || k1 <= 0 || k2 <= 0) return LATER_OK;
  if ((k2 + 63) / 64 > 65535) return LATER_ERR_NOT_SUPPORTED;
  const int mode = out_prec == LATER_PREC_BF16 ? 1 : (out_prec == LATER_PREC_SPLIT3 ? 2 : 0);
  TraceScope trace(s, TRACE_LEAF_GEMM, 2.0 * m * k1 * k2);
  nn_update_kernel<<<dim3((m + NNR - 1) / NNR, (k2 + 63) / 64), 256, 0, s>>>(m, k1, k2, alpha, X, ldx, S, lds, s_trans,
                                                                             lower, Y, ldy, yh, yl, ldh, mode);
  note_launch();
  return cuda_status(cudaGetLastError());
}

later_status_t simt_nn_sub(cudaStream_t s, int m, int k1, int k2, const float* X, int64_t ldx, const float* S,
                           int64_t lds, float* Y, int64_t ldy, void* yh, void* yl, int64_t ldh, int out_prec) {
  return simt_gemm_acc(s, m, k1, k2, -1.f, X, ldx, S, lds, 0, 0, Y, ldy, yh, yl, ldh, out_prec);
}

}  // namespace later

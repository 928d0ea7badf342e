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

namespace later {

namespace {

constexpr int PB = 32;       // panel width
constexpr int BR = 256;      // rows per TSQR block at every level
constexpr int RPL = BR / 32; // rows per lane
constexpr int kGroup = BR / PB;  // blocks of one level stacked into a block of the next (8)
constexpr int APPLY_ROWS = 128;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block MGS of one (<= 256) x 32 block held in registers: 8 warps, warp w
// owns columns 4w .. 4w+3, lane l holds rows l + 32 t (t < 8) of them. Block
// step K: warp K orthonormalises its four columns with MGS using warp
// shuffles only, publishes the four q vectors in shared memory; after one
// barrier every later warp projects its four columns against the four new q
// (16 independent warp reductions in flight). Eight barriers per block
// instead of 32. Columns beyond the block's row count are exactly dependent:
// q = 0 and a zero R row.
constexpr int CPW = 4;  // columns per warp

__device__ __forceinline__ float warp_sum4(float v) { return warp_sum(v); }

__device__ void bmgs_block(float (&a)[CPW][RPL], int mm, float* qbuf /*2 x CPW x BR*/, float* Rs /*32 x 33*/) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll 1
  for (int K = 0; K < PB / CPW; ++K) {
    float* qb = qbuf + (K & 1) * CPW * BR;
    if (w == K) {
#pragma unroll
      for (int j = 0; j < CPW; ++j) {
        const int c = CPW * K + j;
        float ss = 0.f;
#pragma unroll
        for (int t = 0; t < RPL; ++t) ss += a[j][t] * a[j][t];
        ss = warp_sum(ss);
        float nrm = sqrtf(ss);
        if (c >= mm || !(nrm > 0.f)) nrm = 0.f;
        const float inv = nrm > 0.f ? 1.f / nrm : 0.f;
#pragma unroll
        for (int t = 0; t < RPL; ++t) a[j][t] *= inv;
        if (l == 0) Rs[c * 33 + c] = nrm;
        float d[CPW];
#pragma unroll
        for (int jj = 0; jj < CPW; ++jj) {
          d[jj] = 0.f;
          if (jj > j) {
#pragma unroll
            for (int t = 0; t < RPL; ++t) d[jj] += a[j][t] * a[jj][t];
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
          for (int jj = 0; jj < CPW; ++jj)
            if (jj > j) d[jj] += __shfl_xor_sync(0xffffffffu, d[jj], o);
#pragma unroll
        for (int jj = 0; jj < CPW; ++jj)
          if (jj > j) {
#pragma unroll
            for (int t = 0; t < RPL; ++t) a[jj][t] -= d[jj] * a[j][t];
            if (l == 0) Rs[c * 33 + CPW * K + jj] = d[jj];
          }
      }
#pragma unroll
      for (int j = 0; j < CPW; ++j)
#pragma unroll
        for (int t = 0; t < RPL; ++t) qb[j * BR + l + 32 * t] = a[j][t];
    }
    __syncthreads();
    if (w > K) {
      float d[CPW][CPW];  // d[i][j] = q_i . a_j
#pragma unroll
      for (int i = 0; i < CPW; ++i)
#pragma unroll
        for (int j = 0; j < CPW; ++j) d[i][j] = 0.f;
#pragma unroll
      for (int t = 0; t < RPL; ++t) {
#pragma unroll
        for (int i = 0; i < CPW; ++i) {
          const float q = qb[i * BR + l + 32 * t];
#pragma unroll
          for (int j = 0; j < CPW; ++j) d[i][j] += q * a[j][t];
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int i = 0; i < CPW; ++i)
#pragma unroll
          for (int j = 0; j < CPW; ++j) d[i][j] += __shfl_xor_sync(0xffffffffu, d[i][j], o);
#pragma unroll
      for (int t = 0; t < RPL; ++t) {
#pragma unroll
        for (int i = 0; i < CPW; ++i) {
          const float q = qb[i * BR + l + 32 * t];
#pragma unroll
          for (int j = 0; j < CPW; ++j) a[j][t] -= d[i][j] * q;
        }
      }
      if (l < CPW * CPW) {
        const int i = l / CPW, j = l % CPW;
        float v = 0.f;
#pragma unroll
        for (int ii = 0; ii < CPW; ++ii)
#pragma unroll
          for (int jj = 0; jj < CPW; ++jj)
            if (ii == i && jj == j) v = d[ii][jj];
        Rs[(CPW * K + i) * 33 + CPW * w + j] = v;  // R[row of q_i][column of a_j]
      }
    }
  }
  __syncthreads();
}

// Whole TSQR reduction tree in one launch. Each CTA factors one level-0 block;
// the last CTA of each group (atomic ticket) factors the group's stacked R at
// the next level, and so on up to the root. Q factors stay in place.
__global__ void __launch_bounds__(256) tsqr_reduce_kernel(TsqrPlan P) {
  __shared__ float qbuf[2 * CPW * BR];
  __shared__ float Rs[PB * 33];
  __shared__ int last;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  int L = 0;
  int b = blockIdx.x;
  while (true) {
    float* X = P.lev[L];
    const int64_t ld = P.ld[L];
    const int r0 = b * BR;
    const int mm = min(BR, P.rows[L] - r0);
    // Columns at or beyond P.ncols do not exist at level 0 (read as zero, never
    // written); the stacked levels always carry 32 columns.
    const int ncols = (L == 0) ? P.ncols : PB;
    float a[CPW][RPL];
#pragma unroll
    for (int j = 0; j < CPW; ++j)
#pragma unroll
      for (int t = 0; t < RPL; ++t) {
        const int r = l + 32 * t;
        const int col = CPW * w + j;
        a[j][t] = (r < mm && col < ncols) ? __ldcg(&X[r0 + r + static_cast<int64_t>(col) * ld]) : 0.f;
      }
    bmgs_block(a, mm, qbuf, Rs);
#pragma unroll
    for (int j = 0; j < CPW; ++j)
#pragma unroll
      for (int t = 0; t < RPL; ++t) {
        const int r = l + 32 * t;
        const int col = CPW * w + j;
        if (r < mm && col < ncols) X[r0 + r + static_cast<int64_t>(col) * ld] = a[j][t];
      }
    const bool root = (P.nblk[L] == 1);
    float* Ro = root ? P.R : P.lev[L + 1] + 32 * b;
    const int64_t ldo = root ? P.ldr : P.ld[L + 1];
    const int rcols = root ? P.ncols : PB;
    for (int e = threadIdx.x; e < PB * PB; e += blockDim.x) {
      const int i = e % PB, j = e / PB;
      if (i < rcols && j < rcols) Ro[i + static_cast<int64_t>(j) * ldo] = (i <= j) ? Rs[i * 33 + j] : 0.f;
    }
    if (root) break;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      const int g = b / kGroup;
      const int gsize = min(kGroup, P.nblk[L] - kGroup * g);
      int* c = P.counters + P.cnt_off[L] + g;
      const int prev = atomicAdd(c, 1);
      last = (prev == gsize - 1);
      if (last) *c = 0;
    }
    __syncthreads();
    if (!last) break;
    __threadfence();
    b /= kGroup;
    ++L;
  }
}

// Each CTA finishes 256 rows of Q: T = product of its 32x32 path slices
// through the tree, Q = Q0 * T, written in FP32 and as the 16-bit copy.
__global__ void __launch_bounds__(APPLY_ROWS) tsqr_apply_kernel(TsqrPlan P, void* qh, void* ql, int64_t ldh,
                                                                int out_mode) {
  __shared__ float T[PB * 33];
  __shared__ float U[PB * 33];
  const int row0 = blockIdx.x * APPLY_ROWS;
  const int b = row0 / P.br[0];  // level-0 block
  const int tid = threadIdx.x;
  const int top = P.nlev - 1;
  // This thread's row of Q0, loaded before the path composition so the loads overlap it.
  const int row = row0 + tid;
  const bool has_row = row < P.rows[0];
  float* X = P.lev[0];
  const int64_t ld = P.ld[0];
  float q[PB];
#pragma unroll
  for (int k = 0; k < PB; ++k) q[k] = (has_row && k < P.ncols) ? __ldcg(&X[row + static_cast<int64_t>(k) * ld]) : 0.f;
  // Index at level L of the level-0 block b: b / div[L].
  if (top == 0) {
    for (int e = tid; e < PB * PB; e += APPLY_ROWS) T[(e % PB) * 33 + e / PB] = (e % PB == e / PB) ? 1.f : 0.f;
  } else {
    const int bt = b / P.div[top - 1];  // block index at level top-1
    for (int e = tid; e < PB * PB; e += APPLY_ROWS) {
      const int i = e % PB, j = e / PB;
      T[i * 33 + j] = __ldcg(&P.lev[top][32 * bt + i + static_cast<int64_t>(j) * P.ld[top]]);
    }
    for (int L = top - 1; L >= 1; --L) {
      __syncthreads();
      const int bl = b / P.div[L - 1];
      for (int e = tid; e < PB * PB; e += APPLY_ROWS) {  // stage the 32x32 slice
        const int i = e % PB, j = e / PB;
        U[i * 33 + j] = __ldcg(&P.lev[L][32 * bl + i + static_cast<int64_t>(j) * P.ld[L]]);
      }
      __syncthreads();
      constexpr int PER = PB * PB / APPLY_ROWS;
      float out[PER];
#pragma unroll
      for (int u = 0; u < PER; ++u) {
        const int e = tid + APPLY_ROWS * u;
        const int i = e % PB, j = e / PB;
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < PB; ++k) acc += U[i * 33 + k] * T[k * 33 + j];
        out[u] = acc;
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < PER; ++u) {
        const int e = tid + APPLY_ROWS * u;
        T[(e % PB) * 33 + e / PB] = out[u];
      }
    }
  }
  __syncthreads();
  if (!has_row) return;
#pragma unroll 4
  for (int j = 0; j < PB; ++j) {
    if (j >= P.ncols) break;
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

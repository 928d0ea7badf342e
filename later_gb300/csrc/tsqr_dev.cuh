// MGS-TSQR device code shared by the standalone panel kernels (panel.cu) and
// the fused leaf kernel (leaf.cu). Every function here is called by all threads
// of a 256-thread CTA (tsqr_apply_rows: 128 or 256 threads).
//
// The reference factors each 32-column sub-panel with a TSQR tree of
// mgs_kernel2 launches (QR/panel.cu:65-134, 246-325): MGS of every 256-row
// block, the 32x32 R factors stacked and factored again until one block is
// left, then each block's Q multiplied by its slice of the stacked Q.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "panel.cuh"

namespace later {
namespace {

constexpr int PB = 32;       // panel width
constexpr int BR = 256;      // rows per TSQR block at every level
constexpr int RPL = BR / 32; // rows per lane
constexpr int kGroup = BR / PB;  // blocks of one level stacked into a block of the next (8)

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
// Shared memory of tsqr_reduce_block: qbuf (2 * CPW * BR floats), Rs (PB * 33
// floats) and one int. Needs 256 threads; `b` is the level-0 block.
struct TsqrReduceSmem {
  float qbuf[2 * CPW * BR];
  float Rs[PB * 33];
  int last;
};

__device__ void tsqr_reduce_block(const TsqrPlan& P, int b, TsqrReduceSmem& sm) {
  float* qbuf = sm.qbuf;
  float* Rs = sm.Rs;
  int& last = sm.last;
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  int L = 0;
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
    if (root) {
      __syncthreads();
      break;
    }
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
    const bool go = last;
    __syncthreads();  // `last` is read by every thread before the next block may rewrite it
    if (!go) break;
    __threadfence();
    b /= kGroup;
    ++L;
  }
}

// Shared memory of tsqr_apply_rows: two 32 x 33 slices.
struct TsqrApplySmem {
  float T[PB * 33];
  float U[PB * 33];
};

// Finishes rows row0 .. row0 + blockDim.x - 1 of Q (one row per thread, the
// rows inside one level-0 block): T = product of the block's 32x32 path slices
// through the tree, Q = Q0 * T, written in FP32 and as the 16-bit copy.
__device__ void tsqr_apply_rows(const TsqrPlan& P, int row0, void* qh, void* ql, int64_t ldh, int out_mode,
                                TsqrApplySmem& sm) {
  float* T = sm.T;
  float* U = sm.U;
  const int NT = blockDim.x;
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
    for (int e = tid; e < PB * PB; e += NT) T[(e % PB) * 33 + e / PB] = (e % PB == e / PB) ? 1.f : 0.f;
  } else {
    const int bt = b / P.div[top - 1];  // block index at level top-1
    for (int e = tid; e < PB * PB; e += NT) {
      const int i = e % PB, j = e / PB;
      T[i * 33 + j] = __ldcg(&P.lev[top][32 * bt + i + static_cast<int64_t>(j) * P.ld[top]]);
    }
    for (int L = top - 1; L >= 1; --L) {
      __syncthreads();
      const int bl = b / P.div[L - 1];
      for (int e = tid; e < PB * PB; e += NT) {  // stage the 32x32 slice
        const int i = e % PB, j = e / PB;
        U[i * 33 + j] = __ldcg(&P.lev[L][32 * bl + i + static_cast<int64_t>(j) * P.ld[L]]);
      }
      __syncthreads();
      constexpr int MAXPER = PB * PB / 128;  // NT is 128 or 256
      float out[MAXPER];
      const int per = PB * PB / NT;
#pragma unroll
      for (int u = 0; u < MAXPER; ++u) {
        if (u < per) {
          const int e = tid + NT * u;
          const int i = e % PB, j = e / PB;
          float acc = 0.f;
#pragma unroll
          for (int k = 0; k < PB; ++k) acc += U[i * 33 + k] * T[k * 33 + j];
          out[u] = acc;
        }
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < MAXPER; ++u) {
        if (u < per) {
          const int e = tid + NT * u;
          T[(e % PB) * 33 + e / PB] = out[u];
        }
      }
    }
  }
  __syncthreads();
  if (has_row) {
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
  __syncthreads();  // T is reused by the caller's next block
}

}  // namespace
}  // namespace later

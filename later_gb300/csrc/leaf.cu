// Fused rgsqrf leaf: one cooperative launch factors an m x w leaf (w <= 128).
//
// The reference's 128-wide leaf (mgs_caqr_panel_256x128, QR/panel.cu:10-63)
// is four 32-column MGS-TSQR panels glued by six FP32 block-CGS GEMMs, each a
// separate launch, and the panel tree itself is a chain of launches. On GB300
// each of those steps is latency-bound (a 16384 x 32 panel is 2 MB: under a
// microsecond of HBM time), so here the whole leaf is one persistent kernel:
// every CTA owns a fixed slab of rows for the whole leaf and the CTAs meet
// only at grid barriers around deterministic reductions.
//
//   panel (c0, k <= 32), CholQR2:
//     G  = A^T A            slab partials -> barrier -> distributed reduction -> barrier
//                           (panels after the first: G = H - C^T C from the previous
//                           panel's reduction, no reduction of their own)
//     R1 = chol(G)          every CTA, redundantly (bitwise identical), on warp 0
//     Y  = A R1^-1          row-wise substitution on warps 1..7, eight columns behind
//                           the Cholesky (named barrier per group of eight pivots)
//     G2 = Y^T Y            partials -> reduction, together with P = Y^T A_rest
//                           (the later columns) and H = A_next^T A_next
//     R2 = I + F (first order, max|G2 - I| <= 3e-4) or chol(G2); Q = Y R2^-1, R = R2 R1
//     C  = Q^T A_rest       from P locally; R[panel, rest] = C; A_rest -= Q C is applied
//                           by warps 1..7 during the next panel's Cholesky
//   The panel falls back to MGS-TSQR (the reference's algorithm, the tree of
//   tsqr_dev.cuh run over virtual blocks) when chol(G) meets a pivot below
//   1e-4 of its column's squared norm or max|G2 - I| > 1/4; every CTA takes
//   the same decision from the same numbers, and A is not written before it.
//   Its later columns are then projected by separate update steps.
//   With CGS2 the panels keep the recursive order of the reference, glued by
//   update steps (Q cols [c0, c0+w1), A2 cols [c1, c1+w2)):
//     P = Q^T A2 (partials -> reduction, also written into R), A2 -= Q P, twice.
//
// Determinism: the row slabs depend only on m and the grid size; every
// reduction sums the per-CTA partials in CTA order (lane-strided, then a fixed
// shuffle tree), so results are reproducible run to run.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>

#include "dense_dev.cuh"
#include "leaf.cuh"
#include "ptx.cuh"
#include "tsqr_dev.cuh"

namespace later {
namespace {

constexpr int LT = 256;     // threads per CTA
constexpr int GT = 256;     // rows per Gram / substitution tile (one per thread)
constexpr int UT = 64;      // rows per update tile
constexpr int SP = 68;      // row stride of the update tiles (16-byte rows)
constexpr int PART = 8448;  // floats per CTA partial: 64 x 64 (i + 64 j), or a packed 128 x 128 lower triangle
constexpr int kMaxSteps = 8;

struct LeafStep {
  int kind;  // 0: panel (c0, w1 columns); 1: update; 2: panel that also projects columns [c1, c1 + w2)
  int c0, w1, c1, w2;
};

struct LeafPlan {
  int m, w, rpc, nsteps, cgs2, mode, vec, wide;
  LeafStep step[kMaxSteps];
  float* A;
  int64_t lda;
  float* R;
  int64_t ldr;
  char* qh;
  char* ql;
  int64_t ldh;
  float* q1;    // m x 32, ld m
  float* part;  // gridDim.x x PART
  float* red;   // PART
  int* sync;    // arrive, exit, abort
  TsqrPlan tsqr;
  int* status;
  long long budget;
  int* fallbacks;
};

struct PanelSmem {
  float S[32 * (GT + 1)];  // tile of 32 columns x GT rows (column c at c * (GT + 1))
  float G[32 * 33];
  float R1[32 * RCS];  // column-major factors
  float R2[32 * RCS];
  float rinv1[32];
  float rinv2[32];
  int ok;
};

struct UpdateSmem {
  float Qs[UT * SP];
  float As[UT * SP];
  float Ps[64 * SP];
};

union LeafSmem {
  PanelSmem p;
  UpdateSmem u;
  TsqrReduceSmem tr;
  TsqrApplySmem ta;
};

__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// Grid-wide barrier over the co-resident CTAs of a cooperative launch.
// Monotonic arrival counter; every wait is bounded: on timeout the status word
// gets DEV_TIMEOUT, the abort flag is raised and every CTA returns false.
struct GridSync {
  int* arrive;
  int* abort;
  int* status;
  long long budget;
  int epoch;
};

__device__ bool grid_barrier(GridSync& g, int* okflag) {
  __syncthreads();
  ++g.epoch;
  if (threadIdx.x == 0) {
    // Arrive with release semantics (the CTA's writes, ordered before it by
    // __syncthreads, become visible first); poll with relaxed loads, one L2
    // round trip per poll, the abort flag and the clock every eighth poll;
    // then one acquire fence.
    red_release_add(g.arrive, 1);
    const int target = g.epoch * static_cast<int>(gridDim.x);
    const long long t0 = clock64();
    int good = 1;
    for (unsigned it = 1; ld_relaxed(g.arrive) < target; ++it) {
      if ((it & 7) == 0) {
        if (ld_relaxed(g.abort)) {
          good = 0;
          break;
        }
        if (clock64() - t0 > g.budget) {
          report(g.status, DEV_TIMEOUT);
          atomicExch(g.abort, 1);
          good = 0;
          break;
        }
      }
    }
    fence_acq_rel();
    *okflag = good;
  }
  __syncthreads();
  return *okflag != 0;
}

// Copies `total` elements with eight global loads in flight per thread before
// the shared-memory stores (ld(e) -> value, st(e, value)).
template <class Ld, class St>
__device__ __forceinline__ void batched_copy(int total, Ld ld, St st) {
  for (int base = threadIdx.x; base < total; base += 8 * LT) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * LT;
      v[u] = e < total ? ld(e) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * LT;
      if (e < total) st(e, v[u]);
    }
  }
}

// Deterministic reduction of the per-CTA partials over the entries i < ni,
// j < nj (entry i + ld j of every CTA's partial): the entries are split in
// contiguous chunks over the CTAs; a CTA takes 32 entries at a time, one per
// lane, warp w summing the partials of CTAs w, w + 8, ... (eight loads in
// flight), and warp 0 adds the eight warp sums in a fixed order before
// emit(entry, sum).
template <class Emit>
__device__ void reduce_partials(const float* part, int ni, int nj, int ld, Emit emit) {
  __shared__ float ws[8][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int G = static_cast<int>(gridDim.x);
  const int E = ni * nj;
  const int per = (E + G - 1) / G;
  const int e0 = blockIdx.x * per, e1 = min(E, e0 + per);
  for (int base = e0; base < e1; base += 32) {
    const int q = base + lane;
    const bool has = q < e1;
    const int e = has ? (q % ni) + ld * (q / ni) : 0;
    float sum = 0.f;
    for (int c0 = warp; c0 < G; c0 += 64) {  // batches of eight CTAs' partials in flight
      float v[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int c = c0 + 8 * t;
        v[t] = (has && c < G) ? __ldcg(&part[static_cast<int64_t>(c) * PART + e]) : 0.f;
      }
      sum += ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]));
    }
    ws[warp][lane] = sum;
    __syncthreads();
    if (warp == 0 && has) {
      const float t = ((ws[0][lane] + ws[1][lane]) + (ws[2][lane] + ws[3][lane])) +
                      ((ws[4][lane] + ws[5][lane]) + (ws[6][lane] + ws[7][lane]));
      emit(e, t);
    }
    __syncthreads();
  }
}

// Gram partial of the tile in S (32 columns x GT rows): thread (ti, tj) adds
// rows 2ti, 2ti+1 x columns 2tj, 2tj+1 of S^T S into acc.
__device__ __forceinline__ void gram_tile(const float* S, int rows, float (&acc)[2][2]) {
  const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
  const float* x0 = S + (2 * ti) * (GT + 1);
  const float* x1 = x0 + (GT + 1);
  const float* y0 = S + (2 * tj) * (GT + 1);
  const float* y1 = y0 + (GT + 1);
#pragma unroll 8
  for (int r = 0; r < rows; ++r) {
    const float a0 = x0[r], a1 = x1[r], b0 = y0[r], b1 = y1[r];
    acc[0][0] += a0 * b0;
    acc[0][1] += a0 * b1;
    acc[1][0] += a1 * b0;
    acc[1][1] += a1 * b1;
  }
}

__device__ __forceinline__ void write_gram_partial(float* part, const float (&acc)[2][2]) {
  const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
  float* p = part + static_cast<int64_t>(blockIdx.x) * PART;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) p[(2 * ti + a) + 32 * (2 * tj + b)] = acc[a][b];
}

__device__ __forceinline__ void put_shadow(char* hi, char* lo, int64_t o, float v, int mode) {
  if (!hi) return;
  if (mode == 1) {
    reinterpret_cast<__nv_bfloat16*>(hi)[o] = __float2bfloat16_rn(v);
  } else {
    const __half h = __float2half_rn(v);
    reinterpret_cast<__half*>(hi)[o] = h;
    if (mode == 2) reinterpret_cast<__half*>(lo)[o] = __float2half_rn((v - __half2float(h)) * 2048.f);
  }
}

// MGS-TSQR of the panel (the multi-launch path's algorithm) over virtual blocks.
__device__ bool panel_tsqr(const LeafPlan& P, TsqrReduceSmem& tr, TsqrApplySmem& ta, GridSync& gs, int* okflag, int c0,
                           int k) {
  TsqrPlan T = P.tsqr;
  T.lev[0] = P.A + static_cast<int64_t>(c0) * P.lda;
  T.ld[0] = P.lda;
  T.R = P.R + c0 + static_cast<int64_t>(c0) * P.ldr;
  T.ldr = P.ldr;
  T.ncols = k;
  for (int b = blockIdx.x; b < T.nblk[0]; b += gridDim.x) tsqr_reduce_block(T, b, tr);
  if (!grid_barrier(gs, okflag)) return false;
  char* qh = P.qh ? P.qh + static_cast<int64_t>(c0) * P.ldh * 2 : nullptr;
  char* ql = P.ql ? P.ql + static_cast<int64_t>(c0) * P.ldh * 2 : nullptr;
  const int nb = (P.m + BR - 1) / BR;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) tsqr_apply_rows(T, b * BR, qh, ql, P.ldh, P.mode, ta);
  if (blockIdx.x == 0 && threadIdx.x == 0 && P.fallbacks) atomicAdd(P.fallbacks, 1);
  return grid_barrier(gs, okflag);
}

// CholQR2 of columns [c0, c0 + k) over the CTA's slab [r0, r1); false when a
// barrier gave up.
__device__ bool panel_step(const LeafPlan& P, LeafSmem& sm, GridSync& gs, int* okflag, int c0, int k, int r0,
                           int r1) {
  PanelSmem& ps = sm.p;
  const float* Ac = P.A + static_cast<int64_t>(c0) * P.lda;
  const int tid = threadIdx.x;
  // ---- G = A^T A
  {
    float acc[2][2] = {};
    for (int t0 = r0; t0 < r1; t0 += GT) {
      const int rows = min(GT, r1 - t0);
      batched_copy(
          32 * GT,
          [&](int e) {
            const int r = e % GT, c = e / GT;
            return (r < rows && c < k) ? __ldcg(&Ac[t0 + r + static_cast<int64_t>(c) * P.lda]) : 0.f;
          },
          [&](int e, float v) { ps.S[(e / GT) * (GT + 1) + e % GT] = v; });
      __syncthreads();
      gram_tile(ps.S, rows, acc);
      __syncthreads();
    }
    write_gram_partial(P.part, acc);
  }
  if (!grid_barrier(gs, okflag)) return false;
  reduce_partials(P.part, 32, 32, 32, [&](int e, float v) { P.red[e] = v; });
  if (!grid_barrier(gs, okflag)) return false;
  // ---- R1 = chol(G); Q1 = A R1^-1 (scratch); G2 = Q1^T Q1
  for (int e = tid; e < 1024; e += LT) ps.G[(e % 32) * 33 + e / 32] = __ldcg(&P.red[e]);
  __syncthreads();
  chol_upper(ps.G, k, ps.R1, ps.rinv1, false, &ps.ok);
  __syncthreads();
  if (!ps.ok) return panel_tsqr(P, sm.tr, sm.ta, gs, okflag, c0, k);
  {
    float acc[2][2] = {};
    for (int t0 = r0; t0 < r1; t0 += GT) {
      const int rows = min(GT, r1 - t0);
      batched_copy(
          32 * GT,
          [&](int e) {
            const int r = e % GT, c = e / GT;
            return (r < rows && c < k) ? __ldcg(&Ac[t0 + r + static_cast<int64_t>(c) * P.lda]) : 0.f;
          },
          [&](int e, float v) { ps.S[(e / GT) * (GT + 1) + e % GT] = v; });
      __syncthreads();
      if (tid < rows) rows_solve(ps.S, GT + 1, k, tid, ps.R1, ps.rinv1);
      __syncthreads();
      if (tid < rows) {
        for (int j = 0; j < k; ++j) P.q1[t0 + tid + static_cast<int64_t>(j) * P.m] = ps.S[j * (GT + 1) + tid];
      }
      gram_tile(ps.S, rows, acc);
      __syncthreads();
    }
    write_gram_partial(P.part, acc);
  }
  if (!grid_barrier(gs, okflag)) return false;
  reduce_partials(P.part, 32, 32, 32, [&](int e, float v) { P.red[e] = v; });
  if (!grid_barrier(gs, okflag)) return false;
  // ---- R2 = chol(G2) (near the identity); Q = Q1 R2^-1; R = R2 R1
  for (int e = tid; e < 1024; e += LT) ps.G[(e % 32) * 33 + e / 32] = __ldcg(&P.red[e]);
  __syncthreads();
  chol_upper(ps.G, k, ps.R2, ps.rinv2, true, &ps.ok);
  __syncthreads();
  if (!ps.ok) return panel_tsqr(P, sm.tr, sm.ta, gs, okflag, c0, k);
  float* Aw = P.A + static_cast<int64_t>(c0) * P.lda;
  char* qh = P.qh ? P.qh + static_cast<int64_t>(c0) * P.ldh * 2 : nullptr;
  char* ql = P.ql ? P.ql + static_cast<int64_t>(c0) * P.ldh * 2 : nullptr;
  for (int t0 = r0; t0 < r1; t0 += GT) {
    const int rows = min(GT, r1 - t0);
    batched_copy(
        32 * GT,
        [&](int e) {
          const int r = e % GT, c = e / GT;
          return (r < rows && c < k) ? __ldcg(&P.q1[t0 + r + static_cast<int64_t>(c) * P.m]) : 0.f;
        },
        [&](int e, float v) { ps.S[(e / GT) * (GT + 1) + e % GT] = v; });
    __syncthreads();
    if (tid < rows) {
      rows_solve(ps.S, GT + 1, k, tid, ps.R2, ps.rinv2);
      const int r = t0 + tid;
      for (int j = 0; j < k; ++j) {
        const float v = ps.S[j * (GT + 1) + tid];
        Aw[r + static_cast<int64_t>(j) * P.lda] = v;
        put_shadow(qh, ql, r + static_cast<int64_t>(j) * P.ldh, v, P.mode);
      }
    }
    __syncthreads();
  }
  if (blockIdx.x == 0) {
    for (int e = tid; e < 1024; e += LT) {
      const int i = e % 32, j = e / 32;
      if (i < k && j < k) {
        float sum = 0.f;
        for (int l = i; l <= j; ++l) sum += ps.R2[l * RCS + i] * ps.R1[j * RCS + l];
        P.R[(c0 + i) + static_cast<int64_t>(c0 + j) * P.ldr] = i <= j ? sum : 0.f;
      }
    }
  }
  return true;
}

// A2 -= Q (Q^T A2) for Q = columns [c0, c0 + w1), A2 = [c1, c1 + w2) over the
// CTA's slab; the product is written (pass 0) or added (pass 1) into R.
__device__ bool update_step(const LeafPlan& P, LeafSmem& sm, GridSync& gs, int* okflag, const LeafStep& s, int r0,
                            int r1, int pass) {
  UpdateSmem& us = sm.u;
  const float* Q = P.A + static_cast<int64_t>(s.c0) * P.lda;
  float* A2 = P.A + static_cast<int64_t>(s.c1) * P.lda;
  const int tid = threadIdx.x;
  const int ti = tid / 16, tj = tid % 16;
  {
    float acc[4][4] = {};
    for (int t0 = r0; t0 < r1; t0 += UT) {
      const int rows = min(UT, r1 - t0);
      batched_copy(
          UT * 64,
          [&](int e) {
            const int r = e % UT, c = e / UT;
            return (r < rows && c < s.w1) ? __ldcg(&Q[t0 + r + static_cast<int64_t>(c) * P.lda]) : 0.f;
          },
          [&](int e, float v) { us.Qs[(e % UT) * SP + e / UT] = v; });
      batched_copy(
          UT * 64,
          [&](int e) {
            const int r = e % UT, c = e / UT;
            return (r < rows && c < s.w2) ? __ldcg(&A2[t0 + r + static_cast<int64_t>(c) * P.lda]) : 0.f;
          },
          [&](int e, float v) { us.As[(e % UT) * SP + e / UT] = v; });
      __syncthreads();
#pragma unroll 4
      for (int r = 0; r < rows; ++r) {
        const float4 q = *reinterpret_cast<const float4*>(&us.Qs[r * SP + 4 * ti]);
        const float4 a = *reinterpret_cast<const float4*>(&us.As[r * SP + 4 * tj]);
        const float qv[4] = {q.x, q.y, q.z, q.w};
        const float av[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] += qv[u] * av[v];
      }
      __syncthreads();
    }
    float* p = P.part + static_cast<int64_t>(blockIdx.x) * PART;
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) p[(4 * ti + u) + 64 * (4 * tj + v)] = acc[u][v];
  }
  if (!grid_barrier(gs, okflag)) return false;
  reduce_partials(
      P.part, s.w1, s.w2, 64,
      [&](int e, float v) {
        P.red[e] = v;
        float* rp = &P.R[(s.c0 + e % 64) + static_cast<int64_t>(s.c1 + e / 64) * P.ldr];
        *rp = pass ? *rp + v : v;
      });
  if (!grid_barrier(gs, okflag)) return false;
  batched_copy(
      64 * 64,
      [&](int e) { return ((e % 64) < s.w1 && (e / 64) < s.w2) ? __ldcg(&P.red[e]) : 0.f; },
      [&](int e, float v) { us.Ps[(e % 64) * SP + e / 64] = v; });
  for (int t0 = r0; t0 < r1; t0 += UT) {
    const int rows = min(UT, r1 - t0);
    batched_copy(
        UT * 64,
        [&](int e) {
          const int r = e % UT, c = e / UT;
          return (r < rows && c < s.w1) ? __ldcg(&Q[t0 + r + static_cast<int64_t>(c) * P.lda]) : 0.f;
        },
        [&](int e, float v) { us.Qs[(e % UT) * SP + e / UT] = v; });
    __syncthreads();
    // thread (ti, tj): rows 4ti.., columns 4tj..
    float acc[4][4] = {};
    for (int i = 0; i < s.w1; i += 4) {
      float4 q[4], pr[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) q[u] = *reinterpret_cast<const float4*>(&us.Qs[(4 * ti + u) * SP + i]);
#pragma unroll
      for (int l = 0; l < 4; ++l) pr[l] = *reinterpret_cast<const float4*>(&us.Ps[(i + l) * SP + 4 * tj]);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float qv[4] = {q[u].x, q[u].y, q[u].z, q[u].w};
#pragma unroll
        for (int l = 0; l < 4; ++l) {
          acc[u][0] += qv[l] * pr[l].x;
          acc[u][1] += qv[l] * pr[l].y;
          acc[u][2] += qv[l] * pr[l].z;
          acc[u][3] += qv[l] * pr[l].w;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = 4 * ti + u;
      if (r < rows) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const int j = 4 * tj + v;
          if (j < s.w2) {
            float* ap = &A2[t0 + r + static_cast<int64_t>(j) * P.lda];
            *ap = __ldcg(ap) - acc[u][v];
          }
        }
      }
    }
    __syncthreads();
  }
  return true;
}

// ================================================================ resident leaf
// When every CTA's slab is at most RMAX rows, the slab (all w columns) stays
// in shared memory for the whole leaf, column-major with stride XS: one read
// of the leaf from HBM, one write of Q, and every phase in between works on
// shared memory (float4 along rows). The panel's first-pass Q1 goes to a
// separate buffer Y so that the MGS-TSQR fallback still finds the panel as it
// was.
constexpr int RMAX = 256;
constexpr int XS = RMAX + 4;
constexpr int PMS = 100;  // row stride of the 32 x (<= 96) projection block C (16-byte rows)

struct ResPanelSmem {
  float G[32 * 33];
  float R1[32 * RCS];  // column-major factors
  float R2[32 * RCS];
  float rinv1[32];
  float rinv2[32];
  int ok;
  int devbits;  // max |G2 - I| (float bits)
};

constexpr int MS = 132;   // row stride of the leaf-wide Gram / Cholesky factor (16-byte rows)
constexpr int RTS = 132;  // row stride of the 8-row slices of R used by the blocked solves

struct ResSmem {
  float X[kLeafMaxWidth * XS];
  union {
    struct {  // 32-column panels
      float Y[32 * XS];
      float Hn[32 * 33];  // the next panel's Gram matrix before this panel's update (right-looking steps)
      float gp[4096];     // per-row-group partial products
      union {
        struct {
          ResPanelSmem p;
          alignas(16) float Pm[32 * PMS];  // Y^T A_rest, then C = Q^T A_rest (row-major, float4 rows)
        };
        float Ps[64 * SP];  // P = Q^T A2, row-major
        TsqrReduceSmem tr;
        TsqrApplySmem ta;
      };
    };
    struct {  // the whole leaf at once
      float M[kLeafMaxWidth * MS];  // Gram matrix, then L = R^T (lower, row-major) in place; then F
      float Rt[8 * RTS];            // rows b .. b+7 of R (or of F) for the blocked products
      float wrinv[kLeafMaxWidth];
      float gd[kLeafMaxWidth];      // the Gram matrix's diagonal before the factorisation
      int wok;
    };
  };
};

static_assert(sizeof(ResSmem) <= 227 * 1024, "resident leaf shared memory exceeds the per-CTA limit");
static_assert(offsetof(ResSmem, Pm) % 16 == 0 && offsetof(ResSmem, Ps) % 16 == 0 && offsetof(ResSmem, Y) % 16 == 0,
              "float4 tiles need 16-byte alignment");

// Loads rows [r0, r0 + rows) of the leaf's w columns into X; rows [rows, rows rounded up to 4)
// are zeroed (the phases read whole row quads).
__device__ void res_load(const LeafPlan& P, float* X, int r0, int rows, int cols) {
  const int tid = threadIdx.x;
  const int zr = ((rows + 3) & ~3) - rows;
  for (int e = tid; e < zr * cols; e += LT) X[(e / zr) * XS + rows + e % zr] = 0.f;
  if (P.vec) {
    // a column per warp (eight columns in flight), lanes along its row quads (nq <= 64)
    const int nq = rows / 4, warp = tid >> 5, lane = tid & 31;
    for (int cb = warp; cb < cols; cb += 8 * (LT / 32)) {
      for (int qb = 0; qb < nq; qb += 32) {
        const int q = qb + lane;
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int c = cb + u * (LT / 32);
          v[u] = (c < cols && q < nq)
                     ? __ldcg(reinterpret_cast<const float4*>(P.A + r0 + 4 * q + static_cast<int64_t>(c) * P.lda))
                     : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int c = cb + u * (LT / 32);
          if (c < cols && q < nq) *reinterpret_cast<float4*>(&X[c * XS + 4 * q]) = v[u];
        }
      }
    }
    const int tr = rows - 4 * nq;
    for (int e = tid; e < tr * cols; e += LT) {
      const int r = 4 * nq + e % tr, c = e / tr;
      X[c * XS + r] = __ldcg(&P.A[r0 + r + static_cast<int64_t>(c) * P.lda]);
    }
  } else if (rows > 0) {
    batched_copy(
        rows * cols, [&](int e) { return __ldcg(&P.A[r0 + e % rows + static_cast<int64_t>(e / rows) * P.lda]); },
        [&](int e, float v) { X[(e / rows) * XS + e % rows] = v; });
  }
}

// Writes columns [c0, c0 + cols) of the slab back to A (and Q's 16-bit copy when `shadow`).
__device__ void res_store(const LeafPlan& P, const float* X, int r0, int rows, int c0, int cols, bool shadow) {
  // a column per warp, lanes along its rows (row quads when vectorised)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int c = c0 + warp; c < c0 + cols; c += LT / 32) {
    if (P.vec) {
      const int nq = rows / 4;
      for (int q = lane; q < nq; q += 32)
        *reinterpret_cast<float4*>(P.A + r0 + 4 * q + static_cast<int64_t>(c) * P.lda) =
            *reinterpret_cast<const float4*>(&X[c * XS + 4 * q]);
      for (int r = 4 * nq + lane; r < rows; r += 32) P.A[r0 + r + static_cast<int64_t>(c) * P.lda] = X[c * XS + r];
    } else {
      for (int r = lane; r < rows; r += 32) P.A[r0 + r + static_cast<int64_t>(c) * P.lda] = X[c * XS + r];
    }
    if (shadow && P.qh) {
      for (int r = lane; r < rows; r += 32)
        put_shadow(P.qh, P.ql, r0 + r + static_cast<int64_t>(c) * P.ldh, X[c * XS + r], P.mode);
    }
  }
}

// Partial product Xa^T Xb of the slab (Xa = columns [a0, a0 + na) of `Xa`,
// Xb = columns [b0, b0 + nb) of `Xb`, na, nb <= 64) into part (entry i + 64 j).
// Threads form row groups when the output needs fewer than 256 4x4 tiles; the
// groups' sums are added in group order.
// Optional second B buffer: B's columns c >= nb1 are columns b20 + c - nb1 of
// Xb2 (so [Y | X_rest] is one operand); nb up to 128 (at most 256 4x4 tiles).
// Run by threads [t0, t0 + nthr) of the CTA; bar >= 0 names the barrier those
// threads share (else the whole CTA runs it and __syncthreads is used).
template <class Emit>
__device__ void res_tn_emit(const float* Xa, int a0, int na, const float* Xb, int b0, int nb, int rows_eff,
                            float* gp, Emit emit, const float* Xb2 = nullptr, int b20 = 0, int nb1 = 1 << 30,
                            int t0 = 0, int nthr = LT, int bar = -1) {
  const int tid = static_cast<int>(threadIdx.x) - t0;
  const int nta = (na + 3) / 4, ntb = (nb + 3) / 4, nt = nta * ntb;
  const int groups = max(1, nthr / nt);
  const int g = tid / nt, t = tid % nt;
  const int ti = t % nta, tj = t / nta;
  const int npad = 16 * nt;
  if (g < groups) {
    const int chunk = ((rows_eff / 4 + groups - 1) / groups) * 4;
    const int rb = g * chunk, re = min(rows_eff, rb + chunk);
    float acc[4][4] = {};
    // thread (ti, tj) owns columns ti + nta u of Xa and tj + ntb v of Xb: with XS = 4 x odd,
    // the eight float4 rows a warp reads at once fall in eight different bank groups
    const float* pa = Xa + (a0 + ti) * XS;
    const float* pbv[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = tj + ntb * v;  // padded columns (c >= nb) read a valid column; their sums are unused
      pbv[v] = c < nb1 ? Xb + (b0 + c) * XS : Xb2 + min(b20 + c - nb1, kLeafMaxWidth - 1) * XS;
    }
#pragma unroll 2
    for (int r = rb; r < re; r += 4) {
      float4 a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = *reinterpret_cast<const float4*>(&pa[u * nta * XS + r]);
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = *reinterpret_cast<const float4*>(&pbv[v][r]);
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v)
          acc[u][v] = fmaf(a[u].w, b[v].w, fmaf(a[u].z, b[v].z, fmaf(a[u].y, b[v].y, fmaf(a[u].x, b[v].x, acc[u][v]))));
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) gp[g * npad + (ti + nta * u) + 4 * nta * (tj + ntb * v)] = acc[u][v];
  }
  if (bar < 0)
    __syncthreads();
  else
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthr) : "memory");
  // entry e is (e mod 4 nta, e div 4 nta): a shift and a mask when 4 nta is a power of two (na = 32)
  const int w4 = 4 * nta, sh = __ffs(w4) - 1;
  const bool p2 = (w4 & (w4 - 1)) == 0;
  for (int e = tid; e < npad; e += nthr) {
    float s = 0.f;
    for (int gg = 0; gg < groups; ++gg) s += gp[gg * npad + e];
    emit(p2 ? (e & (w4 - 1)) : e % w4, p2 ? (e >> sh) : e / w4, s);
  }
}

// res_tn_emit with the sums written to this CTA's partial block (entry i + 64 j).
__device__ void res_tn(const float* Xa, int a0, int na, const float* Xb, int b0, int nb, int rows_eff, float* gp,
                       float* part) {
  float* p = part + static_cast<int64_t>(blockIdx.x) * PART;
  res_tn_emit(Xa, a0, na, Xb, b0, nb, rows_eff, gp, [&](int i, int j, float v) { p[i + 64 * j] = v; });
}

// Panel fallback: the slab's columns [c0, c0 + k) go back to A, MGS-TSQR runs
// on A (the reference's algorithm), and the factored columns come back.
__device__ bool res_fallback(const LeafPlan& P, ResSmem& S, GridSync& gs, int* okflag, int c0, int k, int r0,
                             int rows) {
  res_store(P, S.X, r0, rows, c0, k, false);
  if (!grid_barrier(gs, okflag)) return false;
  if (!panel_tsqr(P, S.tr, S.ta, gs, okflag, c0, k)) return false;
  for (int e = threadIdx.x; e < rows * k; e += LT) {
    const int r = e % rows, c = c0 + e / rows;
    S.X[c * XS + r] = __ldcg(&P.A[r0 + r + static_cast<int64_t>(c) * P.lda]);
  }
  __syncthreads();
  return true;
}

// D[:, dc + j] = S0[:, sc + j] - sum_{i < K} Sq[:, qc + i] P[i][j] for j < nj
// over the slab's rows (P row-major with stride ldp in shared memory; D may be
// S0). 4 rows x 4 columns per tile, float4 along rows.
__device__ void slab_gemm_sub(float* D, int dc, const float* S0, int sc, const float* Sq, int qc, int K,
                              const float* Pm, int ldp, int nj, int rows_eff, int t0 = -1, int nthr = LT) {
  const int nrt = rows_eff / 4, nct = (nj + 3) / 4;
  for (int t = t0 < 0 ? static_cast<int>(threadIdx.x) : t0; t < nrt * nct; t += nthr) {
    const int rt = t % nrt, ct = t / nrt;
    float acc[4][4] = {};
#pragma unroll 4
    for (int i = 0; i < K; ++i) {
      const float4 q = *reinterpret_cast<const float4*>(&Sq[(qc + i) * XS + 4 * rt]);
      const float4 pp = *reinterpret_cast<const float4*>(&Pm[i * ldp + 4 * ct]);
      const float qv[4] = {q.x, q.y, q.z, q.w};
      const float pv[4] = {pp.x, pp.y, pp.z, pp.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(qv[u], pv[v], acc[u][v]);
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      if (4 * ct + v < nj) {
        const float4 x = *reinterpret_cast<const float4*>(&S0[(sc + 4 * ct + v) * XS + 4 * rt]);
        *reinterpret_cast<float4*>(&D[(dc + 4 * ct + v) * XS + 4 * rt]) =
            make_float4(x.x - acc[0][v], x.y - acc[1][v], x.z - acc[2][v], x.w - acc[3][v]);
      }
    }
  }
}

__device__ bool res_update(const LeafPlan& P, ResSmem& S, GridSync& gs, int* okflag, const LeafStep& s, int rows,
                           int pass);

// After a fallback panel: the columns [rest0, rest0 + nrest) are projected by
// separate update steps (at most 64 columns each).
__device__ bool res_project_rest(const LeafPlan& P, ResSmem& S, GridSync& gs, int* okflag, int c0, int k,
                                 int rest0, int nrest, int rows) {
  for (int j0 = 0; j0 < nrest; j0 += 64) {
    __syncthreads();
    if (!res_update(P, S, gs, okflag, LeafStep{1, c0, k, rest0 + j0, min(64, nrest - j0)}, rows, 0)) return false;
  }
  return true;
}

// Named barriers of the pipelined first pass: warp 0 (the Cholesky) arrives on
// kPubBar + g once pivot group g (eight pivots) is final, one id per group, so
// an arrival can never fall into an earlier group's barrier; warps 1..7 sync
// on it, and on kSolveBar (224 threads) between the phases of each block.
constexpr int kSolveBar = 2, kPubBar = 3, kSolveThreads = LT - 32;  // ids 3 .. 6 for k <= 32

// slab_solve run by warps 1..7 behind the Cholesky on warp 0: block b of
// eight columns starts once pivots b .. b+7 are published.
// First, while the first pivots are computed: the previous panel's deferred
// update of this panel and the later columns, X[:, a0 .. a0 + nsub) -= Q_prev
// C_prev (nsub > 0; Q_prev = the 32 columns before a0, C_prev row-major in
// Cprev), then the partial Gram matrix of the next panel's columns
// [hn0, hn0 + kn) (kn > 0) into hpart[i + 32 j].
__device__ void slab_solve_behind(float* Y, float* X, int a0, int k, int rows, int rows_eff, const float* Rc,
                                  const float* rinv, float* Rt, float* gp, int hn0, int kn, float* hpart, int nsub,
                                  const float* Cprev) {
  const int ct = static_cast<int>(threadIdx.x) - 32;
  if (nsub > 0) {
    slab_gemm_sub(X, a0, X, a0, X, a0 - 32, 32, Cprev, PMS, nsub, rows_eff, ct, kSolveThreads);
    asm volatile("bar.sync %0, %1;" ::"r"(kSolveBar), "r"(kSolveThreads) : "memory");
  }
  if (kn > 0) {
    res_tn_emit(
        X, hn0, kn, X, hn0, kn, rows_eff, gp, [&](int i, int j, float v) { hpart[i + 32 * j] = v; }, nullptr, 0,
        1 << 30, 32, kSolveThreads, kSolveBar);
    asm volatile("bar.sync %0, %1;" ::"r"(kSolveBar), "r"(kSolveThreads) : "memory");  // gp reused later
  }
  for (int b = 0; b < k; b += 8) {
    asm volatile("bar.sync %0, %1;" ::"r"(kPubBar + b / 8), "r"(LT) : "memory");
    for (int r = ct; r < rows_eff; r += kSolveThreads) {
      if (r >= rows) {
        if (b == 0) {
#pragma unroll
          for (int l = 0; l < 8; ++l) Y[l * XS + r] = 0.f;
        }
        continue;
      }
      const float* src = b == 0 ? X + a0 * XS : Y;
      float x[8];
#pragma unroll
      for (int l = 0; l < 8; ++l) x[l] = b + l < k ? src[(b + l) * XS + r] : 0.f;
#pragma unroll
      for (int l = 0; l < 8; ++l) {
        if (b + l < k) {
          x[l] *= rinv[b + l];
#pragma unroll
          for (int j = l + 1; j < 8; ++j) x[j] = fmaf(-x[l], Rc[(b + j) * RCS + b + l], x[j]);
        }
      }
#pragma unroll
      for (int l = 0; l < 8; ++l)
        if (b + l < k) Y[(b + l) * XS + r] = x[l];
    }
    const int nj = k - b - 8;
    if (nj > 0) {
      for (int e = ct; e < 8 * 32; e += kSolveThreads) {
        const int i = e / 32, j = e % 32;
        Rt[i * RCS + j] = (j < nj) ? Rc[(b + 8 + j) * RCS + b + i] : 0.f;
      }
    }
    asm volatile("bar.sync %0, %1;" ::"r"(kSolveBar), "r"(kSolveThreads) : "memory");
    if (nj > 0) {
      if (b == 0)
        slab_gemm_sub(Y, 8, X, a0 + 8, Y, 0, 8, Rt, RCS, nj, rows_eff, ct, kSolveThreads);
      else
        slab_gemm_sub(Y, b + 8, Y, b + 8, Y, b, 8, Rt, RCS, nj, rows_eff, ct, kSolveThreads);
      asm volatile("bar.sync %0, %1;" ::"r"(kSolveBar), "r"(kSolveThreads) : "memory");
    }
  }
}

// One 32-column panel by CholQR2 (first-order second pass when G2 is within
// 3e-4 of I). With nrest > 0 (right-looking steps, full 32-column panel), the
// second reduction also carries P = Y^T A_rest for the leaf's later columns
// [rest0, rest0 + nrest) and H = A_next^T A_next for the next panel's columns
// (the first kn of them, before this panel's update): the projection C =
// Q^T A_rest follows locally, C = (I - F)^T P (first order) or R2^-T P
// (exact), and R[panel, rest] = C. The update A_rest -= Q C is left in Pm for
// the next panel, whose warps 1..7 apply it during its Cholesky (h_in); that
// panel's first-pass Gram matrix is H - C_next^T C_next (the update removes
// exactly the component along the orthonormal Q), so it skips its first
// reduction (*h_out; its second CholQR pass runs on the data as always).
// After a fallback the update is applied at once and *h_out stays false.
__device__ bool res_panel(const LeafPlan& P, ResSmem& S, GridSync& gs, int* okflag, int c0, int k, int r0,
                          int rows, int rest0, int nrest, bool h_in, bool* h_out) {
  ResPanelSmem& ps = S.p;
  const int tid = threadIdx.x;
  const int rows_eff = (rows + 3) & ~3;
  *h_out = false;
  // ---- G = A^T A
  if (h_in) {
    // H - C^T C with C the previous panel's projection block of these columns (rows of Pm):
    // one 2 x 2 tile per thread, float2 reads of C's rows
    {
      const int ti = tid % 16, tj = tid / 16;
      float acc[2][2] = {};
#pragma unroll 8
      for (int l = 0; l < 32; ++l) {
        const float2 a = *reinterpret_cast<const float2*>(&S.Pm[l * PMS + 2 * ti]);
        const float2 b = *reinterpret_cast<const float2*>(&S.Pm[l * PMS + 2 * tj]);
        acc[0][0] = fmaf(a.x, b.x, acc[0][0]);
        acc[0][1] = fmaf(a.x, b.y, acc[0][1]);
        acc[1][0] = fmaf(a.y, b.x, acc[1][0]);
        acc[1][1] = fmaf(a.y, b.y, acc[1][1]);
      }
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int v = 0; v < 2; ++v) {
          const int i = 2 * ti + u, j = 2 * tj + v;
          ps.G[i * 33 + j] = (i < k && j < k) ? S.Hn[i * 33 + j] - acc[u][v] : 0.f;
        }
    }
  } else {
    res_tn(S.X, c0, k, S.X, c0, k, rows_eff, S.gp, P.part);
    if (!grid_barrier(gs, okflag)) return false;
    reduce_partials(P.part, k, k, 64, [&](int e, float v) { P.red[e] = v; });
    if (!grid_barrier(gs, okflag)) return false;
    batched_copy(
        1024, [&](int e) { return ((e % 32) < k && (e / 32) < k) ? __ldcg(&P.red[(e % 32) + 64 * (e / 32)]) : 0.f; },
        [&](int e, float v) { ps.G[(e % 32) * 33 + e / 32] = v; });
  }
  __syncthreads();
  // ---- Cholesky on warp 0; Y = X R1^-1 (rows of the slab) on warps 1..7 behind it,
  // block by block (Y is scratch: a failed factorisation leaves X untouched)
  // (warps 1..7 first compute the next panel's Gram partial, H, in the wait for the first pivots)
  const int kn_next = min(32, nrest);
  float* prt = P.part + static_cast<int64_t>(blockIdx.x) * PART;
  // (h_in: the previous panel left its update of these columns, C_prev in Pm, to this phase)
  if (tid < 32)
    chol_upper(ps.G, k, ps.R1, ps.rinv1, false, &ps.ok, 1e-4f, kPubBar);
  else
    slab_solve_behind(S.Y, S.X, c0, k, rows, rows_eff, ps.R1, ps.rinv1, ps.R2, S.gp, rest0, kn_next,
                      prt + 32 * (32 + nrest), h_in ? k + nrest : 0, S.Pm);
  __syncthreads();
  if (!ps.ok)
    return res_fallback(P, S, gs, okflag, c0, k, r0, rows) &&
           res_project_rest(P, S, gs, okflag, c0, k, rest0, nrest, rows);
  // ---- G2 = Y^T Y (and P = Y^T A_rest)
  if (tid == 0) ps.devbits = 0;
  if (nrest == 0) {
    res_tn(S.Y, 0, k, S.Y, 0, k, rows_eff, S.gp, P.part);
    if (!grid_barrier(gs, okflag)) return false;
    reduce_partials(P.part, k, k, 64, [&](int e, float v) { P.red[e] = v; });
    if (!grid_barrier(gs, okflag)) return false;
    batched_copy(
        1024, [&](int e) { return ((e % 32) < k && (e / 32) < k) ? __ldcg(&P.red[(e % 32) + 64 * (e / 32)]) : 0.f; },
        [&](int e, float v) { ps.G[(e % 32) * 33 + e / 32] = v; });
  } else {
    // partial of [Y^T Y | Y^T A_rest], entry (i, j) at i + 32 j (k = 32)
    // partial of [Y^T Y | Y^T A_rest | A_next^T A_next], entry (i, j) at i + 32 j (k = 32);
    // the A_next^T A_next block was written during the Cholesky
    const int kn = kn_next;
    res_tn_emit(
        S.Y, 0, 32, S.Y, 0, 32 + nrest, rows_eff, S.gp,
        [&](int i, int j, float v) {
          if (j < 32 + nrest) prt[i + 32 * j] = v;  // padded columns would overwrite the H block
        },
        S.X, rest0, 32);
    if (!grid_barrier(gs, okflag)) return false;
    reduce_partials(P.part, 32, 32 + nrest + kn, 32, [&](int e, float v) { P.red[e] = v; });
    if (!grid_barrier(gs, okflag)) return false;
    // all of a thread's loads in flight at once (at most 20: 32 x 160 entries / 256 threads)
    const int nh = 1024 + 32 * nrest, ntot = nh + 32 * kn;
    constexpr int kCp = (32 * 160 + LT - 1) / LT;
    float cv[kCp];
#pragma unroll
    for (int u = 0; u < kCp; ++u) {
      const int e = tid + u * LT;
      cv[u] = e < ntot ? __ldcg(&P.red[e]) : 0.f;
    }
    float dev = 0.f;  // max |G2 - I| (k = 32 here; a NaN counts as a large deviation)
#pragma unroll
    for (int u = 0; u < kCp; ++u) {
      const int e = tid + u * LT;  // e % 32 == tid % 32 for every u
      if (e < 1024) {
        ps.G[(e % 32) * 33 + e / 32] = cv[u];
        const float d = fabsf(cv[u] - ((e % 32) == (e / 32) ? 1.f : 0.f));
        dev = d <= dev ? dev : (d == d ? d : 1.f);
      } else if (e < nh) {
        S.Pm[(e % 32) * PMS + (e - 1024) / 32] = cv[u];
      } else if (e < ntot) {
        S.Hn[(e % 32) * 33 + (e - nh) / 32] = cv[u];
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dev = fmaxf(dev, __shfl_xor_sync(0xffffffffu, dev, o));
    if ((tid & 31) == 0) atomicMax(&ps.devbits, __float_as_int(dev));
  }
  __syncthreads();
  // G2 = I + E. When max |E| <= 3e-4, chol(I + E) = I + F + O(E^2) with
  // F = triu(E) - diag(E) / 2, and Q = Y (I - F) has Q^T Q = I + O(E^2) and
  // Q (I + F) R1 = Y R1 + O(E^2): no second Cholesky and no second
  // substitution chain, only a small product. Otherwise the exact path.
  // max |E| over all threads (a NaN entry counts as a large deviation); the
  // fused path took it while copying G2.
  if (nrest == 0) {
    float dev = 0.f;
    for (int e = tid; e < 1024; e += LT) {
      const int i = e / 32, j = e % 32;
      if (i < k && j < k) {
        const float d = fabsf(ps.G[i * 33 + j] - (i == j ? 1.f : 0.f));
        dev = d <= dev ? dev : (d == d ? d : 1.f);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dev = fmaxf(dev, __shfl_xor_sync(0xffffffffu, dev, o));
    if ((tid & 31) == 0) atomicMax(&ps.devbits, __float_as_int(dev));
  }
  __syncthreads();
  const bool first_order = __int_as_float(ps.devbits) <= 3e-4f;
  if (first_order) {
    // F row-major (stride RCS) in R2's place
    for (int e = tid; e < 32 * RCS; e += LT) {
      const int i = e / RCS, j = e % RCS;
      float f = 0.f;
      if (i < k && j < k && i <= j) f = i == j ? 0.5f * (ps.G[i * 33 + i] - 1.f) : ps.G[i * 33 + j];
      ps.R2[e] = f;
    }
    __syncthreads();
    slab_gemm_sub(S.X, c0, S.Y, 0, S.Y, 0, k, ps.R2, RCS, k, rows_eff);
  } else {
    chol_upper(ps.G, k, ps.R2, ps.rinv2, true, &ps.ok);
    __syncthreads();
    if (!ps.ok)
      return res_fallback(P, S, gs, okflag, c0, k, r0, rows) &&
             res_project_rest(P, S, gs, okflag, c0, k, rest0, nrest, rows);
    // ---- Q = Y R2^-1 into the slab
    if (tid < rows) rows_solve(S.Y, XS, k, tid, ps.R2, ps.rinv2);
    __syncthreads();
    for (int e = tid; e < k * rows_eff; e += LT) {
      const int c = e / rows_eff, r = e % rows_eff;
      if (r < rows) S.X[(c0 + c) * XS + r] = S.Y[c * XS + r];
    }
  }
  if (nrest > 0) {
    // C = Q^T A_rest from P = Y^T A_rest. First order: C = (I - F)^T P = P - F^T P
    // (F upper, row-major in R2) as 4 x 4 tiles, one per thread (8 x 24 at most),
    // written back over P after a barrier. Exact: C = R2^-T P (R2 column-major),
    // forward substitution per column in place.
    const int nct = (nrest + 3) / 4;
    const int it = tid % 8, jt = tid / 8;
    const bool mine = first_order && tid < 8 * nct;
    float cv[4][4];
    if (mine) {
      float acc[4][4] = {};
#pragma unroll 4
      for (int l = 0; l < 32; ++l) {
        const float4 f = *reinterpret_cast<const float4*>(&ps.R2[l * RCS + 4 * it]);
        const float4 q = *reinterpret_cast<const float4*>(&S.Pm[l * PMS + 4 * jt]);
        const float fv[4] = {f.x, f.y, f.z, f.w};
        const float qv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(fv[u], qv[v], acc[u][v]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float4 q = *reinterpret_cast<const float4*>(&S.Pm[(4 * it + u) * PMS + 4 * jt]);
        cv[u][0] = q.x - acc[u][0];
        cv[u][1] = q.y - acc[u][1];
        cv[u][2] = q.z - acc[u][2];
        cv[u][3] = q.w - acc[u][3];
      }
    }
    if (!first_order) {
      for (int j = tid; j < nrest; j += LT) {
        for (int i = 0; i < 32; ++i) {
          float v = S.Pm[i * PMS + j];
          for (int l = 0; l < i; ++l) v = fmaf(-ps.R2[i * RCS + l], S.Pm[l * PMS + j], v);
          S.Pm[i * PMS + j] = v * ps.rinv2[i];
        }
      }
    }
    __syncthreads();
    if (mine) {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        *reinterpret_cast<float4*>(&S.Pm[(4 * it + u) * PMS + 4 * jt]) =
            make_float4(cv[u][0], cv[u][1], cv[u][2], cv[u][3]);
    }
    __syncthreads();
    const int n = 32 * nrest;
    // R[panel, rest] = C (spread over the CTAs); A_rest -= Q C is left to the next
    // panel's Cholesky phase (warps 1..7), which reads C from Pm
    for (int e = static_cast<int>(blockIdx.x) * LT + tid; e < n; e += static_cast<int>(gridDim.x) * LT)
      P.R[(c0 + e % 32) + static_cast<int64_t>(rest0 + e / 32) * P.ldr] = S.Pm[(e % 32) * PMS + e / 32];
    *h_out = true;
  }
  // R = R2 R1 (exact) or (I + F) R1 (first order); every CTA holds both
  // factors, the 1024 entries go to the first four CTAs (one per thread)
  {
    for (int e = static_cast<int>(blockIdx.x) * LT + tid; e < 1024; e += static_cast<int>(gridDim.x) * LT) {
      const int i = e % 32, j = e / 32;
      if (i < k && j < k) {
        float sum = 0.f;
        if (first_order) {
          sum = ps.R1[j * RCS + i];
          for (int l = i; l <= j; ++l) sum = fmaf(ps.R2[i * RCS + l], ps.R1[j * RCS + l], sum);
        } else {
          for (int l = i; l <= j; ++l) sum += ps.R2[l * RCS + i] * ps.R1[j * RCS + l];
        }
        P.R[(c0 + i) + static_cast<int64_t>(c0 + j) * P.ldr] = i <= j ? sum : 0.f;
      }
    }
  }
  __syncthreads();
  return true;
}

__device__ bool res_update(const LeafPlan& P, ResSmem& S, GridSync& gs, int* okflag, const LeafStep& s, int rows,
                           int pass) {
  const int rows_eff = (rows + 3) & ~3;
  res_tn(S.X, s.c0, s.w1, S.X, s.c1, s.w2, rows_eff, S.gp, P.part);
  if (!grid_barrier(gs, okflag)) return false;
  reduce_partials(
      P.part, s.w1, s.w2, 64,
      [&](int e, float v) {
        P.red[e] = v;
        float* rp = &P.R[(s.c0 + e % 64) + static_cast<int64_t>(s.c1 + e / 64) * P.ldr];
        *rp = pass ? *rp + v : v;
      });
  if (!grid_barrier(gs, okflag)) return false;
  batched_copy(
      64 * 64, [&](int e) { return ((e % 64) < s.w1 && (e / 64) < s.w2) ? __ldcg(&P.red[e]) : 0.f; },
      [&](int e, float v) { S.Ps[(e % 64) * SP + e / 64] = v; });
  __syncthreads();
  // A2 -= Q P
  slab_gemm_sub(S.X, s.c1, S.X, s.c1, S.X, s.c0, s.w1, S.Ps, SP, s.w2, rows_eff);
  __syncthreads();
  return true;
}

// ------------------------------------------------------------- leaf-wide CholQR2
// In place lower Cholesky M = L L^T of the n x n matrix in M (row-major, stride
// ms, multiple of 4; n <= 128), all 256 threads: right-looking in blocks of 4
// columns. Thread 0 factors the 4 x 4 diagonal block (pivots d * rsqrt(d), the
// reciprocal pivots into rinv), one thread per row solves the block column
// below it, and the CTA applies the rank-4 update to the trailing lower
// triangle, 8 rows x 1 column per work item with float4 reads of the L rows.
// *okout = 0 on a pivot below ratio * gd[k] (gd: the diagonal before the
// factorisation) or a non-finite value.
__device__ void chol_cta(float* M, int ms, int n, const float* gd, float ratio, float* rinv, int* okout) {
  const int tid = threadIdx.x;
  if (tid == 0) *okout = 1;
  for (int kb = 0; kb < n; kb += 4) {
    const int kw = min(4, n - kb);
    __syncthreads();
    if (tid == 0) {
      int ok = *okout;
      for (int a = 0; a < kw; ++a) {
        float* ra = M + (kb + a) * ms + kb;
        float d = ra[a];
        for (int b = 0; b < a; ++b) d = fmaf(-ra[b], ra[b], d);
        if (!(d > ratio * gd[kb + a]) || !(d < 3.0e38f)) {
          ok = 0;
          d = 1.f;
        }
        const float ri = rsqrtf(d);
        ra[a] = d * ri;
        rinv[kb + a] = ri;
        for (int c = a + 1; c < kw; ++c) {
          float* rc = M + (kb + c) * ms + kb;
          float v = rc[a];
          for (int b = 0; b < a; ++b) v = fmaf(-rc[b], ra[b], v);
          rc[a] = v * ri;
        }
      }
      *okout = ok;
    }
    __syncthreads();
    const int t0 = kb + kw, nt = n - t0;
    if (tid < nt) {  // block column below the diagonal block
      float* ri_ = M + (t0 + tid) * ms + kb;
      for (int a = 0; a < kw; ++a) {
        const float* ra = M + (kb + a) * ms + kb;
        float v = ri_[a];
        for (int b = 0; b < a; ++b) v = fmaf(-ri_[b], ra[b], v);
        ri_[a] = v * rinv[kb + a];
      }
    }
    __syncthreads();
    if (nt > 0) {  // trailing lower triangle: M[i][j] -= L[i][kb..] . L[j][kb..], t0 <= j <= i < n
      // thread = (column j, row parity): no index arithmetic beyond a shift, rows i >= j
      const int j = tid >> 1, par = tid & 1;
      if (j < nt) {
        const float4 lj = *reinterpret_cast<const float4*>(&M[(t0 + j) * ms + kb]);
#pragma unroll 4
        for (int i = j + par; i < nt; i += 2) {
          const float4 li = *reinterpret_cast<const float4*>(&M[(t0 + i) * ms + kb]);
          float* mij = &M[(t0 + i) * ms + t0 + j];
          *mij = fmaf(-li.w, lj.w, fmaf(-li.z, lj.z, fmaf(-li.y, lj.y, fmaf(-li.x, lj.x, *mij))));
        }
      }
    }
  }
  __syncthreads();
}

// Packed lower-triangle partial G = X^T X of the slab's first w columns (entry
// i (i + 1) / 2 + j for j <= i) into part. 4 x 4 tiles over the tile grid's
// upper half (tile (ti, tj), ti <= tj, columns ti + nt u and tj + nt v: each
// unordered pair once), float4 along rows.
__device__ void wide_gram(const float* X, int w, int rows_eff, float* part) {
  const int nt = (w + 3) / 4;
  const int ntiles = nt * (nt + 1) / 2;
  float* p = part + static_cast<int64_t>(blockIdx.x) * PART;
  for (int t = threadIdx.x; t < ntiles; t += LT) {
    int ti = static_cast<int>((sqrtf(8.f * t + 1.f) - 1.f) * 0.5f);
    while (ti * (ti + 1) / 2 > t) --ti;
    while ((ti + 1) * (ti + 2) / 2 <= t) ++ti;
    const int tj = t - ti * (ti + 1) / 2;  // tj <= ti
    const float* pa = X + tj * XS;
    const float* pb = X + ti * XS;
    float acc[4][4] = {};
#pragma unroll 2
    for (int r = 0; r < rows_eff; r += 4) {
      float4 a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = *reinterpret_cast<const float4*>(&pa[u * nt * XS + r]);
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = *reinterpret_cast<const float4*>(&pb[v * nt * XS + r]);
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v)
          acc[u][v] = fmaf(a[u].w, b[v].w, fmaf(a[u].z, b[v].z, fmaf(a[u].y, b[v].y, fmaf(a[u].x, b[v].x, acc[u][v]))));
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int cj = tj + nt * u, ci = ti + nt * v;  // columns of a and b
        const int i = max(ci, cj), j = min(ci, cj);
        if (i < w && (ti != tj || ci >= cj)) p[i * (i + 1) / 2 + j] = acc[u][v];
      }
  }
}

// Loads the reduced packed Gram matrix: diagonal into gd; off-diagonal entries
// into M's lower triangle (M[i][j], i > j) or, with `upper`, into its upper
// triangle (M[j][i]) so that a factor already held in the lower triangle stays.
__device__ void wide_load_gram(const float* red, int w, float* M, float* gd, bool upper) {
  const int E = w * (w + 1) / 2;
  batched_copy(
      E, [&](int e) { return __ldcg(&red[e]); },
      [&](int e, float v) {
        int i = static_cast<int>((sqrtf(8.f * e + 1.f) - 1.f) * 0.5f);
        while (i * (i + 1) / 2 > e) --i;
        while ((i + 1) * (i + 2) / 2 <= e) ++i;
        const int j = e - i * (i + 1) / 2;
        if (i == j) {
          gd[i] = v;
          if (!upper) M[i * MS + i] = v;
        } else {
          M[upper ? j * MS + i : i * MS + j] = v;
        }
      });
}

// X R = A in place for the slab's first w columns (R upper, R[i][j] = L[j][i] =
// M[j * MS + i]; rinv its reciprocal pivots): blocks of 8 columns, the 8 x 8
// diagonal block per row (a chain of 8), the later columns as a tiled product.
__device__ void wide_solve(float* X, int w, int rows, int rows_eff, const float* M, const float* rinv, float* Rt) {
  const int tid = threadIdx.x;
  for (int b = 0; b < w; b += 8) {
    if (tid < rows) {
      float x[8];
#pragma unroll
      for (int l = 0; l < 8; ++l) x[l] = b + l < w ? X[(b + l) * XS + tid] : 0.f;
#pragma unroll
      for (int l = 0; l < 8; ++l) {
        if (b + l < w) {
          x[l] *= rinv[b + l];
#pragma unroll
          for (int j = l + 1; j < 8; ++j)
            if (b + j < w) x[j] = fmaf(-x[l], M[(b + j) * MS + b + l], x[j]);
        }
      }
#pragma unroll
      for (int l = 0; l < 8; ++l)
        if (b + l < w) X[(b + l) * XS + tid] = x[l];
    }
    const int nj = w - b - 8;
    if (nj > 0) {
      for (int e = tid; e < 8 * nj; e += LT) {
        const int i = e / nj, j = e % nj;
        Rt[i * RTS + j] = M[(b + 8 + j) * MS + b + i];  // R[b + i][b + 8 + j]
      }
    }
    __syncthreads();
    if (nj > 0) {
      slab_gemm_sub(X, b + 8, X, b + 8, X, b, 8, Rt, RTS, nj, rows_eff);
      __syncthreads();
    }
  }
}

// X <- X (I - F) in place, F upper: F[i][j] = M[i * MS + j] for i < j, F[i][i] =
// fd[i]. Column blocks of 8 from the last to the first, so the columns a block
// reads are still the old ones: each row takes its block's own 8 x 8 triangle
// in registers, the columns before the block are applied as one tiled product
// (F's block column staged row-major, stride 8, in Ft), then the triangle.
__device__ void wide_apply_f(float* X, int w, int rows, int rows_eff, const float* M, const float* fd, float* Ft) {
  const int tid = threadIdx.x;
  for (int b = ((w - 1) / 8) * 8; b >= 0; b -= 8) {
    const int nb = min(8, w - b);
    float dpart[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) dpart[j] = 0.f;
    if (tid < rows) {
      float x[8];
#pragma unroll
      for (int l = 0; l < 8; ++l) x[l] = l < nb ? X[(b + l) * XS + tid] : 0.f;
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int l = 0; l <= j; ++l)
          if (j < nb) dpart[j] = fmaf(x[l], l == j ? fd[b + j] : M[(b + l) * MS + b + j], dpart[j]);
    }
    for (int e = tid; e < b * 8; e += LT) {
      const int i = e / 8, j = e % 8;
      Ft[i * 8 + j] = j < nb ? M[i * MS + b + j] : 0.f;
    }
    __syncthreads();
    if (b > 0) {
      slab_gemm_sub(X, b, X, b, X, 0, b, Ft, 8, nb, rows_eff);
      __syncthreads();
    }
    if (tid < rows) {
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (j < nb) X[(b + j) * XS + tid] -= dpart[j];
    }
    __syncthreads();
  }
}

// The whole leaf by CholQR2 at once. Returns 1 when done (Q in the slab, R in
// P.R), 0 when the leaf is not conditioned well enough for it (nothing has been
// written; the caller reloads the slab and factors the leaf by 32-column
// panels), -1 when a grid barrier gave up.
__device__ int res_wide(const LeafPlan& P, ResSmem& S, GridSync& gs, int* okflag, int rows) {
  const int tid = threadIdx.x;
  const int w = P.w;
  const int rows_eff = (rows + 3) & ~3;
  const int E = w * (w + 1) / 2;
  auto put = [&](int e, float v) { P.red[e] = v; };
  // ---- pass 1: G = X^T X, L = chol(G) (lower triangle of M), X <- X R1^-1
  wide_gram(S.X, w, rows_eff, P.part);
  if (!grid_barrier(gs, okflag)) return -1;
  reduce_partials(P.part, E, 1, E, put);
  if (!grid_barrier(gs, okflag)) return -1;
  wide_load_gram(P.red, w, S.M, S.gd, false);
  __syncthreads();
  chol_cta(S.M, MS, w, S.gd, 1e-4f, S.wrinv, &S.wok);
  if (!S.wok) return 0;
  wide_solve(S.X, w, rows, rows_eff, S.M, S.wrinv, S.Rt);
  // ---- pass 2: G2 = X^T X = I + E into M's upper triangle (L stays below)
  wide_gram(S.X, w, rows_eff, P.part);
  if (!grid_barrier(gs, okflag)) return -1;
  reduce_partials(P.part, E, 1, E, put);
  if (!grid_barrier(gs, okflag)) return -1;
  wide_load_gram(P.red, w, S.M, S.gd, true);
  __syncthreads();
  if (tid < 32) {  // first order only when max |E| <= 3e-4
    float dev = 0.f;
    for (int i = tid; i < w; i += 32) {
      dev = fmaxf(dev, fabsf(S.gd[i] - 1.f));
      for (int j = i + 1; j < w; ++j) dev = fmaxf(dev, fabsf(S.M[i * MS + j]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dev = fmaxf(dev, __shfl_xor_sync(0xffffffffu, dev, o));
    if (tid == 0) S.wok = dev <= 3e-4f ? 1 : 0;
  }
  __syncthreads();
  if (!S.wok) return 0;
  for (int i = tid; i < w; i += LT) S.gd[i] = 0.5f * (S.gd[i] - 1.f);  // F's diagonal
  __syncthreads();
  // ---- Q = X (I - F); R = (I + F) R1
  wide_apply_f(S.X, w, rows, rows_eff, S.M, S.gd, S.Rt);
  // R = (I + F) R1: every CTA holds the same L and F, so column j of R is formed
  // by CTA j mod grid, one row per thread (R1[l][j] = L[j][l] is row j of M)
  for (int j = blockIdx.x; j < w; j += gridDim.x) {
    for (int i = tid; i < w; i += LT) {
      float sum = 0.f;
      if (i <= j) {
        sum = S.M[j * MS + i];  // R1[i][j]
        sum = fmaf(S.gd[i], S.M[j * MS + i], sum);
        for (int l = i + 1; l <= j; ++l) sum = fmaf(S.M[i * MS + l], S.M[j * MS + l], sum);
      }
      P.R[i + static_cast<int64_t>(j) * P.ldr] = sum;
    }
  }
  __syncthreads();
  return 1;
}

__global__ void __launch_bounds__(LT, 1) leaf_res_kernel(LeafPlan P) {
  extern __shared__ __align__(16) unsigned char smraw[];
  ResSmem& S = *reinterpret_cast<ResSmem*>(smraw);
  __shared__ int okflag;
  GridSync gs{P.sync, P.sync + 2, P.status, P.budget, 0};
  const int r0 = min(P.m, static_cast<int>(blockIdx.x) * P.rpc);
  const int rows = min(P.m, r0 + P.rpc) - r0;
  res_load(P, S.X, r0, rows, P.w);
  __syncthreads();
  bool ok = true;
  int done = 0;
  if (P.wide) {
    done = res_wide(P, S, gs, &okflag, rows);
    if (done < 0) ok = false;
    if (done == 0) {  // not conditioned well enough for one CholQR2 over the leaf: 32-column panels
      __syncthreads();
      res_load(P, S.X, r0, rows, P.w);
      __syncthreads();
    }
  }
  bool h_ready = false;  // the next panel's first-pass Gram matrix is already in smem
  for (int i = 0; i < P.nsteps && ok && !done; ++i) {
    const LeafStep s = P.step[i];
    __syncthreads();
    if (s.kind == 0 || s.kind == 2) {
      bool h_next = false;
      ok = res_panel(P, S, gs, &okflag, s.c0, s.w1, r0, rows, s.c1, s.kind == 2 ? s.w2 : 0, h_ready, &h_next);
      h_ready = h_next;
    } else {
      ok = res_update(P, S, gs, &okflag, s, rows, 0);
      if (ok && P.cgs2) ok = res_update(P, S, gs, &okflag, s, rows, 1);
    }
  }
  __syncthreads();
  griddep_launch();  // the next kernel (a trailing update) may be scheduled as these CTAs finish
  if (ok) res_store(P, S.X, r0, rows, 0, P.w, true);
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const int prev = atomicAdd(P.sync + 1, 1);
    if (prev == static_cast<int>(gridDim.x) - 1) {
      atomicExch(P.sync, 0);
      atomicExch(P.sync + 2, 0);
      atomicExch(P.sync + 1, 0);
    }
  }
}

__global__ void __launch_bounds__(LT, 1) leaf_kernel(LeafPlan P) {
  extern __shared__ __align__(16) unsigned char smraw[];
  LeafSmem& sm = *reinterpret_cast<LeafSmem*>(smraw);
  __shared__ int okflag;
  GridSync gs{P.sync, P.sync + 2, P.status, P.budget, 0};
  const int r0 = min(P.m, static_cast<int>(blockIdx.x) * P.rpc);
  const int r1 = min(P.m, r0 + P.rpc);
  for (int i = 0; i < P.nsteps; ++i) {
    const LeafStep s = P.step[i];
    bool ok = true;
    __syncthreads();  // the phases share one shared-memory union: the previous step's readers are done
    if (s.kind == 0) {
      ok = panel_step(P, sm, gs, &okflag, s.c0, s.w1, r0, r1);
    } else {
      ok = update_step(P, sm, gs, &okflag, s, r0, r1, 0);
      __syncthreads();
      if (ok && P.cgs2) ok = update_step(P, sm, gs, &okflag, s, r0, r1, 1);
    }
    if (!ok) break;
  }
  // Exit protocol: the last CTA out resets the counters for the next launch.
  __syncthreads();
  griddep_launch();
  if (threadIdx.x == 0) {
    __threadfence();
    const int prev = atomicAdd(P.sync + 1, 1);
    if (prev == static_cast<int>(gridDim.x) - 1) {
      atomicExch(P.sync, 0);
      atomicExch(P.sync + 2, 0);
      atomicExch(P.sync + 1, 0);
    }
  }
}

// Right-looking steps for the resident kernel without CGS2: one step per
// 32-column panel, each projecting all later columns of the leaf.
void build_steps_rl(int w, LeafPlan* P) {
  for (int c0 = 0; c0 < w; c0 += 32) {
    const int k = std::min(32, w - c0);
    P->step[P->nsteps++] = LeafStep{2, c0, k, c0 + k, w - c0 - k};
  }
}

void build_steps(int w, int c0, LeafPlan* P) {
  if (w <= 32) {
    P->step[P->nsteps++] = LeafStep{0, c0, w, 0, 0};
    return;
  }
  const int w1 = ((w / 32 + 1) / 2) * 32, w2 = w - w1;  // split_half
  build_steps(w1, c0, P);
  P->step[P->nsteps++] = LeafStep{1, c0, w1, c0 + w1, w2};
  build_steps(w2, c0 + w1, P);
}

// Resident-kernel grid for m rows, or 0 when a slab would exceed RMAX rows or
// the device cannot hold one CTA per SM with the resident shared memory.
int leaf_res_grid(int m, int* rpc) {
  static int cached[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  // spread the rows over every SM (the phases' time scales with the slab height,
  // the grid barriers do not), in slabs of a multiple of 4 rows, at most RMAX
  *rpc = static_cast<int>(round_up((m + num_sms() - 1) / num_sms(), 4));
  if (*rpc > RMAX) return 0;
  const int g = (m + *rpc - 1) / *rpc;
  int per_sm = dev < 64 ? cached[dev] : 0;
  if (per_sm == 0) {
    if (cudaFuncSetAttribute(leaf_res_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(sizeof(ResSmem))) != cudaSuccess)
      return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, leaf_res_kernel, LT, sizeof(ResSmem)) != cudaSuccess)
      return 0;
    if (per_sm < 1) per_sm = -1;
    if (dev < 64) cached[dev] = per_sm;
  }
  return per_sm > 0 ? g : 0;
}

int leaf_grid(int m) {
  static int cached[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  int per_sm = 0;
  if (dev < 64 && cached[dev]) {
    per_sm = cached[dev];
  } else {
    if (cudaFuncSetAttribute(leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(sizeof(LeafSmem))) != cudaSuccess)
      return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, leaf_kernel, LT, sizeof(LeafSmem)) != cudaSuccess)
      return 0;
    if (dev < 64) cached[dev] = per_sm;
  }
  if (per_sm < 1) return 0;
  const int g = std::min(num_sms(), (m + 63) / 64);
  return std::max(1, g);
}

}  // namespace

int64_t leaf_fused_work(int m) {
  TsqrPlan plan{};
  int ncnt = 0;
  int64_t stack = 0;
  tsqr_plan_sizes(m, &plan, &stack, &ncnt);
  return static_cast<int64_t>(m) * 32 + static_cast<int64_t>(num_sms()) * PART + PART + stack +
         64 * (kMaxTsqrLevels + 4);
}

later_status_t leaf_fused(cudaStream_t st, int m, int w, float* A, int64_t lda, float* R, int64_t ldr, void* qh,
                          void* ql, int64_t ldh, int out_prec, int cgs2, bool try_wide, Arena& ws, int* sync,
                          int* tsqr_counters, long long budget, int* fallbacks) {
  if (w < 1 || w > kLeafMaxWidth || m < w) return LATER_ERR_INVALID_ARG;
  int res_rpc = 0;
  const int res_grid = leaf_res_grid(m, &res_rpc);
  const bool resident = res_grid > 0;
  const int grid = resident ? res_grid : leaf_grid(m);
  if (grid < 1) return LATER_ERR_NOT_SUPPORTED;
  LeafPlan P{};
  P.m = m;
  P.w = w;
  P.rpc = resident ? res_rpc : (m + grid - 1) / grid;
  P.vec = (reinterpret_cast<uintptr_t>(A) % 16 == 0) && (lda % 4 == 0);
  // one CholQR2 over the whole leaf first (resident slabs, wider than one panel, no CGS2 requested)
  P.wide = try_wide && resident && w > 32 && !cgs2;
  P.cgs2 = cgs2;
  P.mode = out_prec == LATER_PREC_BF16 ? 1 : (out_prec == LATER_PREC_SPLIT3 ? 2 : 0);
  if (resident && !cgs2)
    build_steps_rl(w, &P);
  else
    build_steps(w, 0, &P);
  P.A = A;
  P.lda = lda;
  P.R = R;
  P.ldr = ldr;
  P.qh = static_cast<char*>(qh);
  P.ql = static_cast<char*>(ql);
  P.ldh = ldh;
  P.sync = sync;
  P.status = device_status_ptr();
  P.budget = budget > 0 ? budget : kDefaultBudgetCycles;
  P.fallbacks = fallbacks;
  // fallback tree over an m-row panel
  int64_t stack = 0;
  int ncnt = 0;
  tsqr_plan_sizes(m, &P.tsqr, &stack, &ncnt);
  if (P.tsqr.nblk[P.tsqr.nlev - 1] != 1 || ncnt > 2048) return LATER_ERR_NOT_SUPPORTED;
  const size_t mark = ws.used();
  P.q1 = ws.take<float>(static_cast<size_t>(m) * 32);
  P.part = ws.take<float>(static_cast<size_t>(grid) * PART);
  P.red = ws.take<float>(PART);
  for (int L = 1; L < P.tsqr.nlev; ++L) {
    P.tsqr.ld[L] = round_up(P.tsqr.rows[L], 64);
    P.tsqr.lev[L] = ws.take<float>(P.tsqr.ld[L] * 32);
  }
  if (ws.failed() || !P.q1 || !P.part || !P.red) {
    ws.reset(mark);
    return LATER_ERR_WORKSPACE;
  }
  P.tsqr.counters = tsqr_counters;
  P.tsqr.status = P.status;
  P.tsqr.budget = P.budget;
  if (ws.sizing()) {
    ws.reset(mark);
    return LATER_OK;
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(LT);
  cfg.dynamicSmemBytes = resident ? sizeof(ResSmem) : sizeof(LeafSmem);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  TraceScope trace(st, TRACE_PANEL);
  const cudaError_t e = resident ? cudaLaunchKernelEx(&cfg, leaf_res_kernel, P) : cudaLaunchKernelEx(&cfg, leaf_kernel, P);
  note_launch();
  ws.reset(mark);
  return cuda_status(e);
}

}  // namespace later

// Small dense factorisations shared by the fused rgsqrf leaf (leaf.cu) and the
// Cholesky / triangular-solve leaves (blas3.cu): compact-code kernels run by
// one warp or one thread per row, where instruction-cache pressure and the
// dependency chain, not arithmetic, set the time.
#pragma once
#include <cuda_runtime.h>

namespace later {
namespace {

constexpr int RCS = 36;  // stride of the column-major 32 x 32 R factors in shared memory (16-byte columns)

// Upper Cholesky G = R^T R of the k x k matrix in G (stride 33) by warp 0,
// written as compact code (runtime loops): it runs once per panel on one warp,
// so what matters is the instruction count per pivot. Lane i carries the
// residual of row i in a register window d[j] = G[i][kb + j] that shifts left
// by four columns per block step. A block step factors four pivots (the 4 x 4
// diagonal block through shuffles), publishes the four new columns of L as one
// float4 per lane in shared memory, and applies the rank-4 update to the
// window with one float4 load per column. Pivots are d * rsqrt(d) (the factor
// only has to be used consistently: CholQR2 applies exactly the R it
// computed). Writes R column-major, Rc[j * RCS + i] = R[i][j] (zeros outside
// the k x k upper triangle), and rinv[i] = rsqrt of the i-th pivot, 1 / R[i][i]
// to within an ulp. Fails (*okout = 0) on a pivot below 1e-4 of its column's
// original diagonal, a non-finite value, or, with `near_identity`,
// max |G - I| > 1/4.
// With pub_bar >= 0, warp 0 also arrives on named barrier pub_bar + g
// (counting pub_count threads, default blockDim.x) once pivots 8g .. 8g + 7 are final (R rows and
// rinv published; the last group may be partial): ceil(k / 8) arrivals, one
// per barrier id, so other warps can consume R block by block. Each id is
// used once per call: the caller separates calls by a full-block barrier.
__device__ __forceinline__ void chol_upper(const float* G, int k, float* Rc, float* rinv, bool near_identity,
                                           int* okout, float ratio = 1e-4f, int pub_bar = -1, int pub_count = 0) {
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  float* Lb = Rc;  // scratch for the published block columns reuses Rc's layout: Lb[lane * RCS + kb .. kb+3]
  float d[32];
  float dev = 0.f;
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const float g = (lane < k && j < k) ? G[lane * 33 + j] : 0.f;
    d[j] = j <= lane ? g : 0.f;
    if (lane < k && j < k) dev = fmaxf(dev, fabsf(g - (j == lane ? 1.f : 0.f)));
  }
  bool ok = true;
  if (near_identity) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dev = fmaxf(dev, __shfl_xor_sync(0xffffffffu, dev, o));
    if (!(dev <= 0.25f)) ok = false;
  }
  const float gdiag = lane < k ? G[lane * 33 + lane] : 1.f;
  for (int kb = 0; kb < k; kb += 4) {
    // four pivots of the block: lane i's L[i][kb + b] in l[b]
    float l[4];
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int kk = kb + b;
      float lb = 0.f;
      if (kk < k) {  // warp-uniform
        float dk = __shfl_sync(0xffffffffu, d[b], kk);
        const float gk = __shfl_sync(0xffffffffu, gdiag, kk);
        if (!(dk > ratio * gk) || !(dk < 3.0e38f)) {
          ok = false;
          dk = 1.f;
        }
        const float ri = rsqrtf(dk);
        lb = lane == kk ? dk * ri : ((lane > kk && lane < k) ? d[b] * ri : 0.f);
        if (lane == kk) rinv[kk] = ri;
        // update the rest of the block's four columns inside the window
#pragma unroll
        for (int c = b + 1; c < 4; ++c) {
          const float lc = __shfl_sync(0xffffffffu, lb, kb + c < 32 ? kb + c : 0);
          if (kb + c <= lane) d[c] -= lb * lc;
        }
      }
      l[b] = lb;
    }
    *reinterpret_cast<float4*>(&Lb[lane * RCS + kb]) = make_float4(l[0], l[1], l[2], l[3]);
    __syncwarp();
    if (pub_bar >= 0 && ((kb + 4) % 8 == 0 || kb + 4 >= k))
      asm volatile("bar.arrive %0, %1;" ::"r"(pub_bar + kb / 8),
                   "r"(pub_count > 0 ? pub_count : static_cast<int>(blockDim.x))
                   : "memory");
    // rank-4 update of the window columns kb + 4 .. and shift by four
#pragma unroll
    for (int j = 4; j < 32; ++j) {
      const int c = kb + j;
      float nv = d[j];
      if (c < 32) {
        const float4 lc = *reinterpret_cast<const float4*>(&Lb[c * RCS + kb]);  // L[c][kb .. kb+3]
        if (c <= lane) nv = fmaf(-l[3], lc.w, fmaf(-l[2], lc.z, fmaf(-l[1], lc.y, fmaf(-l[0], lc.x, nv))));
      }
      d[j - 4] = nv;
    }
#pragma unroll
    for (int j = 28; j < 32; ++j) d[j] = 0.f;
    __syncwarp();
  }
  // Rc already holds L[i][j] at i * RCS + j = R[j][i] for j < k (rounded up to a
  // multiple of 4, zeros beyond k); clear the rest of the 32 x 32 factor.
  for (int j = (k + 3) & ~3; j < 32; ++j) Rc[lane * RCS + j] = 0.f;
  if (lane == 0) *okout = ok ? 1 : 0;
  __syncwarp();
}

// One eight-column group b of rows_solve: columns b .. b + 7 of row r are
// solved (the 8 x 8 diagonal block in registers) and removed from the later
// columns b + 8 .. k - 1 (R read as float4 pairs). Needs R's rows b .. b + 7.
__device__ __forceinline__ void rows_solve_group(float* X, int ld, int k, int r, const float* Rc, const float* rinv,
                                                 int b) {
  {
    float x[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) x[l] = b + l < k ? X[(b + l) * ld + r] : 0.f;
#pragma unroll
    for (int l = 0; l < 8; ++l) {
      if (b + l < k) {
        x[l] *= rinv[b + l];
#pragma unroll
        for (int j = l + 1; j < 8; ++j) x[j] -= x[l] * Rc[(b + j) * RCS + b + l];
      }
    }
#pragma unroll
    for (int l = 0; l < 8; ++l)
      if (b + l < k) X[(b + l) * ld + r] = x[l];
#pragma unroll 4
    for (int j = b + 8; j < k; ++j) {
      const float4 r0 = *reinterpret_cast<const float4*>(&Rc[j * RCS + b]);
      const float4 r1 = *reinterpret_cast<const float4*>(&Rc[j * RCS + b + 4]);
      float t = X[j * ld + r];
      t = fmaf(-x[0], r0.x, t);
      t = fmaf(-x[1], r0.y, t);
      t = fmaf(-x[2], r0.z, t);
      t = fmaf(-x[3], r0.w, t);
      t = fmaf(-x[4], r1.x, t);
      t = fmaf(-x[5], r1.y, t);
      t = fmaf(-x[6], r1.z, t);
      t = fmaf(-x[7], r1.w, t);
      X[j * ld + r] = t;
    }
  }
}

// x R = a for row r of the k columns X[c * ld + r], c < k, in place (R upper
// k x k column-major in Rc, rinv its reciprocal pivots), eight columns at a time.
__device__ __forceinline__ void rows_solve(float* X, int ld, int k, int r, const float* Rc, const float* rinv) {
  for (int b = 0; b < k; b += 8) rows_solve_group(X, ld, k, r, Rc, rinv, b);
}

}  // namespace
}  // namespace later

// Batched QR of many independent tall-skinny FP32 matrices of uneven sizes in
// one persistent-kernel launch (no reference counterpart; the comparator is a
// loop of later_rgsqrf calls, one per matrix).
//
// Plan (host, once per batch shape): descriptors sorted by decreasing cost
// 2 n^2 m (longest first, so the largest matrices start first and the small
// ones fill the tail), uploaded to device memory. Run (capturable in a CUDA
// graph: one counter reset + one launch): every CTA of a persistent grid
// (CTAs-per-SM x SM count) takes the next matrix from an atomic work queue and
// factors it alone:
//   for each 32-column panel p (left-looking):
//     CGS2:  C = Q_<p^T A_p ; A_p -= Q_<p C   (twice; R[<p, p] = C1 + C2)
//     CholQR2 inside the panel: G = A_p^T A_p, G = L L^T (one warp),
//            A_p <- A_p L^-T   (twice; R[p, p] = L2^T L1^T)
// Every product streams the matrix through shared memory in row chunks of
// CR rows (the tunable tile), five streams per panel with the products that
// share a chunk fused, and needs no inter-CTA communication. All arithmetic is FP32; reductions run in
// a fixed order (deterministic). A Cholesky pivot <= 0 (a rank-deficient or
// very ill-conditioned panel: CholQR2 needs kappa(panel) below about 1e3 in
// FP32) marks that matrix's status as LATER_ERR_NUMERIC.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "../../include/later_c.h"
#include "runtime.cuh"

namespace later {

namespace {

constexpr int PW = 32;        // panel width
constexpr int NMAX = 256;     // widest matrix
constexpr int THREADS = 256;

struct Item {
  float* A;
  float* R;
  int64_t lda, ldr;
  int m, n;
  int idx;  // position in the caller's list (for the status array)
  int pad;
};

// Shared tiles are column-major (column c at c * (CR + 4)) so that four
// consecutive rows of a column are one float4.
template <int CR>
struct Smem {
  static constexpr int LD = CR + 4;
  float q[(NMAX - PW) * LD];  // chunk of the previous Q columns (up to 224)
  float a[PW * LD];           // chunk of the current panel
  float c[(NMAX - PW) * (PW + 1)];  // projection coefficients C[i][j]
  float g[PW][PW + 1];              // Gram matrix / Cholesky factor
  float ginv[PW];                   // reciprocals of the factor's diagonal
  float red[8 * PW * PW];           // per-warp partial sums of a Gram matrix
};

// Stages rows [r0, r0 + rows) of columns [c0, c0 + nc) into dst (column-major,
// stride LD), rows beyond `rows` (up to the next multiple of 4) as zeros.
// Global reads are issued eight per thread before the shared-memory stores
// (float4 along rows when the matrix allows it), so a chunk costs a few memory
// latencies rather than one per element.
template <int CR>
__device__ void stage(float* dst, const Item& it, int r0, int rows, int c0, int nc) {
  const int LD = CR + 4;
  const int rq = (rows + 3) & ~3;
  const bool vec = rows == rq && (it.lda % 4 == 0) && (reinterpret_cast<uintptr_t>(it.A) % 16 == 0);
  if (vec) {  // r0 is a multiple of CR, so every float4 is aligned
    // (column, row quad) of element e: a shift when nq is a power of two (every full chunk), which
    // spares the integer divisions that otherwise dominate the staging
    const int nq = rq / 4, total = nq * nc;
    const bool p2 = (nq & (nq - 1)) == 0;
    const int sh = __ffs(nq) - 1;
    for (int base = threadIdx.x; base < total; base += 8 * THREADS) {
      float4 v[8];
      int off[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = base + u * THREADS;
        const int c = p2 ? e >> sh : e / nq, q = e - c * nq;
        off[u] = c * LD + 4 * q;
        v[u] = e < total ? *reinterpret_cast<const float4*>(it.A + r0 + 4 * q + static_cast<int64_t>(c0 + c) * it.lda)
                         : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (base + u * THREADS < total) *reinterpret_cast<float4*>(&dst[off[u]]) = v[u];
    }
    return;
  }
  const int total = rq * nc;
  for (int base = threadIdx.x; base < total; base += 8 * THREADS) {
    float v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * THREADS;
      const int r = e % rq, c = e / rq;
      v[u] = (e < total && r < rows) ? it.A[r0 + r + static_cast<int64_t>(c0 + c) * it.lda] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = base + u * THREADS;
      if (e < total) dst[(e / rq) * LD + e % rq] = v[u];
    }
  }
}

// ---- chunk-level pieces (the staged chunk: Q columns in s.q, the panel in s.a)

// acc[u] += sum over the chunk's rows of Q[r][i0 + 8u] A[r][j] (thread j = t % 32,
// i0 = t / 32): the Q column read as one float4 (the same for the whole warp: a
// broadcast), the A column as one float4.
template <int CR>
__device__ __forceinline__ void chunk_project(const Smem<CR>& s, int rq, int k1, float (&acc)[(NMAX - PW) / 8]) {
  const int LD = CR + 4;
  const int j = threadIdx.x % PW, i0 = threadIdx.x / PW;
  for (int r = 0; r < rq; r += 4) {
    const float4 av = *reinterpret_cast<const float4*>(&s.a[j * LD + r]);
#pragma unroll
    for (int u = 0; u < (NMAX - PW) / 8; ++u) {
      if (i0 + 8 * u < k1) {
        const float4 qv = *reinterpret_cast<const float4*>(&s.q[(i0 + 8 * u) * LD + r]);
        acc[u] = fmaf(qv.w, av.w, fmaf(qv.z, av.z, fmaf(qv.y, av.y, fmaf(qv.x, av.x, acc[u]))));
      }
    }
  }
}

// C (k1 x w) from the projection accumulators into s.c (zeros for j >= w).
template <int CR>
__device__ __forceinline__ void store_projection(Smem<CR>& s, int k1, int w, const float (&acc)[(NMAX - PW) / 8]) {
  const int j = threadIdx.x % PW, i0 = threadIdx.x / PW;
#pragma unroll
  for (int u = 0; u < (NMAX - PW) / 8; ++u)
    if (i0 + 8 * u < k1) s.c[(i0 + 8 * u) * (PW + 1) + j] = (j < w) ? acc[u] : 0.f;
}

// The staged panel chunk -= Q C (C in s.c): each thread updates a 4-row x
// 2-column tile, reading Q as float4 along rows.
template <int CR>
__device__ __forceinline__ void chunk_subtract(Smem<CR>& s, int rq, int k1) {
  const int LD = CR + 4;
  const int nr4 = rq / 4, ntile = nr4 * (PW / 2);
  const bool p2 = (nr4 & (nr4 - 1)) == 0;
  const int sh = __ffs(nr4) - 1;
  for (int e = threadIdx.x; e < ntile; e += THREADS) {
    const int ct = p2 ? e >> sh : e / nr4, rt = e - ct * nr4;
    const int r = 4 * rt, jj = 2 * ct;
    float4 x0 = *reinterpret_cast<const float4*>(&s.a[jj * LD + r]);
    float4 x1 = *reinterpret_cast<const float4*>(&s.a[(jj + 1) * LD + r]);
    for (int i = 0; i < k1; ++i) {
      const float4 qv = *reinterpret_cast<const float4*>(&s.q[i * LD + r]);
      const float c0v = s.c[i * (PW + 1) + jj], c1v = s.c[i * (PW + 1) + jj + 1];
      x0.x = fmaf(-qv.x, c0v, x0.x); x0.y = fmaf(-qv.y, c0v, x0.y);
      x0.z = fmaf(-qv.z, c0v, x0.z); x0.w = fmaf(-qv.w, c0v, x0.w);
      x1.x = fmaf(-qv.x, c1v, x1.x); x1.y = fmaf(-qv.y, c1v, x1.y);
      x1.z = fmaf(-qv.z, c1v, x1.z); x1.w = fmaf(-qv.w, c1v, x1.w);
    }
    *reinterpret_cast<float4*>(&s.a[jj * LD + r]) = x0;
    *reinterpret_cast<float4*>(&s.a[(jj + 1) * LD + r]) = x1;
  }
}

// acc += the Gram matrix of a staged panel chunk (column-major at a): warp wp takes rows 4 wp,
// 4 wp + 32, ...; lane (ti = l % 8, tj = l / 8) owns entries (ti + 8u, tj + 4v).
template <int CR>
__device__ __forceinline__ void chunk_gram(const float* a, int rq, float (&acc)[4][8]) {
  const int LD = CR + 4;
  const int lane = threadIdx.x % 32, wp = threadIdx.x / 32;
  const int ti = lane % 8, tj = lane / 8;
  for (int r = 4 * wp; r < rq; r += 32) {
    float4 x[4], y[8];
#pragma unroll
    for (int u = 0; u < 4; ++u) x[u] = *reinterpret_cast<const float4*>(&a[(ti + 8 * u) * LD + r]);
#pragma unroll
    for (int v = 0; v < 8; ++v) y[v] = *reinterpret_cast<const float4*>(&a[(tj + 4 * v) * LD + r]);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 8; ++v)
        acc[u][v] = fmaf(x[u].w, y[v].w, fmaf(x[u].z, y[v].z, fmaf(x[u].y, y[v].y, fmaf(x[u].x, y[v].x, acc[u][v]))));
  }
}

// G (w x w, into s.g) from the per-warp Gram accumulators, added in warp order.
template <int CR>
__device__ __forceinline__ void store_gram(Smem<CR>& s, int w, const float (&acc)[4][8]) {
  const int lane = threadIdx.x % 32, wp = threadIdx.x / 32;
  const int ti = lane % 8, tj = lane / 8;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) s.red[wp * PW * PW + (ti + 8 * u) * PW + tj + 4 * v] = acc[u][v];
  __syncthreads();
  for (int e = threadIdx.x; e < PW * PW; e += THREADS) {
    float v = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) v += s.red[q * PW * PW + e];
    const int i = e / PW, j = e % PW;
    s.g[i][j] = (i < w && j < w) ? v : 0.f;
  }
  __syncthreads();
}

// M = L^-T (upper, into s.c as M[i][j] at i * (PW + 1) + j) for L = s.g (lower,
// reciprocal diagonal in s.ginv), by warp 0: lane j solves L x = e_j by forward
// substitution, x being column j of L^-1, i.e. row j of M.
template <int CR>
__device__ __forceinline__ void invert_factor(Smem<CR>& s, int w) {
  if (threadIdx.x < 32) {
    const int j = threadIdx.x;
    float x[PW];
#pragma unroll
    for (int i = 0; i < PW; ++i) {
      float v = (i == j) ? 1.f : 0.f;
#pragma unroll
      for (int k = 0; k < i; ++k) v = fmaf(-s.g[i][k], x[k], v);
      x[i] = (i >= j && i < w) ? v * s.ginv[i] : 0.f;
    }
#pragma unroll
    for (int i = 0; i < PW; ++i) s.c[j * (PW + 1) + i] = x[i];
  }
  __syncthreads();
}

// out = in M (the staged chunk times the upper triangular M = L^-T, columns < w):
// each thread computes a 4-row tile of the column pair (ct, PW - 1 - ct), so
// every thread does the same number of multiply-adds.
template <int CR>
__device__ __forceinline__ void chunk_solve(const Smem<CR>& s, const float* in, float* out, int rq, int w) {
  const int LD = CR + 4;
  const int nr4 = rq / 4, ntile = nr4 * (PW / 2);
  const bool p2 = (nr4 & (nr4 - 1)) == 0;
  const int sh = __ffs(nr4) - 1;
  for (int e = threadIdx.x; e < ntile; e += THREADS) {
    const int ct = p2 ? e >> sh : e / nr4, rt = e - ct * nr4;
    const int r = 4 * rt, ja = ct, jb = PW - 1 - ct;
    float4 xa = make_float4(0.f, 0.f, 0.f, 0.f), xb = xa;
    const int ea = min(ja + 1, w), eb = min(jb + 1, w);
    int i = 0;
    for (; i < ea; ++i) {
      const float4 v = *reinterpret_cast<const float4*>(&in[i * LD + r]);
      const float ma = s.c[i * (PW + 1) + ja], mb = s.c[i * (PW + 1) + jb];
      xa.x = fmaf(v.x, ma, xa.x); xa.y = fmaf(v.y, ma, xa.y); xa.z = fmaf(v.z, ma, xa.z); xa.w = fmaf(v.w, ma, xa.w);
      xb.x = fmaf(v.x, mb, xb.x); xb.y = fmaf(v.y, mb, xb.y); xb.z = fmaf(v.z, mb, xb.z); xb.w = fmaf(v.w, mb, xb.w);
    }
    for (; i < eb; ++i) {
      const float4 v = *reinterpret_cast<const float4*>(&in[i * LD + r]);
      const float mb = s.c[i * (PW + 1) + jb];
      xb.x = fmaf(v.x, mb, xb.x); xb.y = fmaf(v.y, mb, xb.y); xb.z = fmaf(v.z, mb, xb.z); xb.w = fmaf(v.w, mb, xb.w);
    }
    *reinterpret_cast<float4*>(&out[ja * LD + r]) = xa;
    *reinterpret_cast<float4*>(&out[jb * LD + r]) = xb;
  }
}

// A staged panel chunk (column-major at a) back to rows [r0, r0 + rows) of
// columns [c0, c0 + w) of A.
template <int CR>
__device__ __forceinline__ void chunk_store(const float* a, const Item& it, int r0, int rows, int c0, int w) {
  const int LD = CR + 4;
  // a column per warp, lanes along its rows (no integer division per element)
  for (int jj = threadIdx.x / 32; jj < w; jj += THREADS / 32)
    for (int r = threadIdx.x % 32; r < rows; r += 32)
      it.A[r0 + r + static_cast<int64_t>(c0 + jj) * it.lda] = a[jj * LD + r];
}

// In-place lower Cholesky of s.g (w x w) by warp 0; returns false on a pivot <= 0.
template <int CR>
__device__ bool chol(Smem<CR>& s, int w) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
    for (int k = 0; k < w; ++k) {
      float d = s.g[k][k];
      if (!(d > 0.f)) {
        if (l == 0) bad = 1;
        d = 1.f;
      }
      const float piv = sqrtf(d);
      __syncwarp();
      if (l == k) {
        s.g[k][k] = piv;
        s.ginv[k] = 1.f / piv;
      }
      if (l > k && l < w) s.g[l][k] /= piv;
      __syncwarp();
      if (l > k && l < w)
        for (int i = l; i < w; ++i) s.g[i][l] -= s.g[i][k] * s.g[l][k];
      __syncwarp();
    }
  }
  __syncthreads();
  return bad == 0;
}

// One matrix, panel by panel (left-looking), in five streams of row chunks per
// panel, each fusing the products that share a staged chunk:
//   1. C1 = Q^T A_p
//   2. A_p -= Q C1, then C2 = Q^T A_p on the updated chunk
//   3. A_p -= Q C2, then G1 = A_p^T A_p          (the first panel: G1 alone)
//   4. A_p <- A_p L1^-T, then G2 = A_p^T A_p     (G1 = L1 L1^T)
//   5. A_p <- A_p L2^-T                          (G2 = L2 L2^T)
// R[<p, p] = C1 + C2, R[p, p] = L2^T L1^T.
template <int CR>
__global__ void __launch_bounds__(THREADS, 1) batched_qr_kernel(const Item* items, int count, int* queue, int* status) {
  extern __shared__ float smraw[];
  Smem<CR>& s = *reinterpret_cast<Smem<CR>*>(smraw);
  __shared__ int cur;
  __shared__ float r1[PW][PW + 1];  // first CholQR factor (R1 = L1^T)
  while (true) {
    if (threadIdx.x == 0) cur = atomicAdd(queue, 1);
    __syncthreads();
    const int k = cur;
    __syncthreads();
    if (k >= count) break;
    const Item it = items[k];
    bool ok = true;
    // R starts at zero (upper factor with zeros below the diagonal).
    for (int e = threadIdx.x; e < it.n * it.n; e += THREADS)
      it.R[e % it.n + static_cast<int64_t>(e / it.n) * it.ldr] = 0.f;
    for (int c0 = 0; c0 < it.n; c0 += PW) {
      const int w = min(PW, it.n - c0);
      const int k1 = c0;  // previous Q columns
      {
        float gacc[4][8] = {};
        if (k1 > 0) {
          // Stream 1: C1.
          float acc[(NMAX - PW) / 8] = {};
          for (int r0 = 0; r0 < it.m; r0 += CR) {
            const int rows = min(CR, it.m - r0), rq = (rows + 3) & ~3;
            __syncthreads();
            stage<CR>(s.q, it, r0, rows, 0, k1);
            stage<CR>(s.a, it, r0, rows, c0, w);
            __syncthreads();
            chunk_project(s, rq, k1, acc);
          }
          __syncthreads();
          store_projection(s, k1, w, acc);
          __syncthreads();
          for (int e = threadIdx.x; e < k1 * w; e += THREADS) {
            const int i = e % k1, j = e / k1;
            it.R[i + static_cast<int64_t>(c0 + j) * it.ldr] = s.c[i * (PW + 1) + j];
          }
          // Stream 2: A_p -= Q C1, C2 on the updated chunk.
#pragma unroll
          for (int u = 0; u < (NMAX - PW) / 8; ++u) acc[u] = 0.f;
          for (int r0 = 0; r0 < it.m; r0 += CR) {
            const int rows = min(CR, it.m - r0), rq = (rows + 3) & ~3;
            __syncthreads();
            stage<CR>(s.q, it, r0, rows, 0, k1);
            stage<CR>(s.a, it, r0, rows, c0, w);
            __syncthreads();
            chunk_subtract(s, rq, k1);
            __syncthreads();
            chunk_project(s, rq, k1, acc);
            chunk_store<CR>(s.a, it, r0, rows, c0, w);
          }
          __syncthreads();
          store_projection(s, k1, w, acc);
          __syncthreads();
          for (int e = threadIdx.x; e < k1 * w; e += THREADS) {
            const int i = e % k1, j = e / k1;
            it.R[i + static_cast<int64_t>(c0 + j) * it.ldr] += s.c[i * (PW + 1) + j];
          }
          // Stream 3: A_p -= Q C2, G1.
          for (int r0 = 0; r0 < it.m; r0 += CR) {
            const int rows = min(CR, it.m - r0), rq = (rows + 3) & ~3;
            __syncthreads();
            stage<CR>(s.q, it, r0, rows, 0, k1);
            stage<CR>(s.a, it, r0, rows, c0, w);
            __syncthreads();
            chunk_subtract(s, rq, k1);
            __syncthreads();
            chunk_gram<CR>(s.a, rq, gacc);
            chunk_store<CR>(s.a, it, r0, rows, c0, w);
          }
        } else {
          for (int r0 = 0; r0 < it.m; r0 += CR) {
            const int rows = min(CR, it.m - r0), rq = (rows + 3) & ~3;
            __syncthreads();
            stage<CR>(s.a, it, r0, rows, c0, w);
            __syncthreads();
            chunk_gram<CR>(s.a, rq, gacc);
          }
        }
        __syncthreads();
        store_gram(s, w, gacc);
      }
      ok &= chol(s, w);
      invert_factor(s, w);
      for (int e = threadIdx.x; e < PW * PW; e += THREADS) {
        const int i = e % PW, j = e / PW;  // R1 = L1^T: R1[i][j] = L1[j][i], i <= j
        r1[i][j] = (i <= j && j < w) ? s.g[j][i] : 0.f;
      }
      // Stream 4: A_p <- A_p L1^-T, G2 (the solved chunk goes to s.q, free here).
      {
        float gacc[4][8] = {};
        for (int r0 = 0; r0 < it.m; r0 += CR) {
          const int rows = min(CR, it.m - r0), rq = (rows + 3) & ~3;
          __syncthreads();
          stage<CR>(s.a, it, r0, rows, c0, w);
          __syncthreads();
          chunk_solve(s, s.a, s.q, rq, w);
          __syncthreads();
          chunk_gram<CR>(s.q, rq, gacc);
          chunk_store<CR>(s.q, it, r0, rows, c0, w);
        }
        __syncthreads();
        store_gram(s, w, gacc);
      }
      ok &= chol(s, w);
      invert_factor(s, w);
      // Stream 5: A_p <- A_p L2^-T.
      for (int r0 = 0; r0 < it.m; r0 += CR) {
        const int rows = min(CR, it.m - r0), rq = (rows + 3) & ~3;
        __syncthreads();
        stage<CR>(s.a, it, r0, rows, c0, w);
        __syncthreads();
        chunk_solve(s, s.a, s.q, rq, w);
        __syncthreads();
        chunk_store<CR>(s.q, it, r0, rows, c0, w);
      }
      // R[p,p] = L2^T R1 (upper x upper).
      for (int e = threadIdx.x; e < w * w; e += THREADS) {
        const int i = e % w, j = e / w;
        float v = 0.f;
        if (i <= j)
          for (int q = i; q <= j; ++q) v += s.g[q][i] * r1[q][j];  // L2^T[i][q] = L2[q][i]
        it.R[c0 + i + static_cast<int64_t>(c0 + j) * it.ldr] = v;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0 && status) status[it.idx] = ok ? 0 : LATER_ERR_NUMERIC;
  }
}

template <int CR>
later_status_t launch(const Item* items, int count, int* queue, int* status, int ctas_per_sm, cudaStream_t st) {
  const size_t smem = sizeof(Smem<CR>);
  static bool done[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !done[dev]) {
    LATER_CHECK_CUDA(cudaFuncSetAttribute(batched_qr_kernel<CR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(smem)));
    done[dev] = true;
  }
  LATER_CHECK_CUDA(cudaMemsetAsync(queue, 0, sizeof(int), st));
  TraceScope trace(st, TRACE_PANEL);
  batched_qr_kernel<CR><<<num_sms() * ctas_per_sm, THREADS, smem, st>>>(items, count, queue, status);
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace

// Tile variants the autotuner chooses among: rows per streamed chunk x CTAs per SM.
int batched_variants() { return 4; }
void batched_variant(int v, int* chunk_rows, int* ctas_per_sm) {
  static const int cr[4] = {32, 64, 32, 64};
  static const int cps[4] = {1, 1, 2, 2};
  *chunk_rows = cr[v & 3];
  *ctas_per_sm = cps[v & 3];
}

int64_t batched_plan_bytes(int count) { return static_cast<int64_t>(count) * sizeof(Item) + 256; }

later_status_t batched_plan(cudaStream_t st, int count, const later_qr_item_t* host_items, void* plan,
                            int64_t plan_bytes) {
  if (count < 1 || !host_items || !plan) return LATER_ERR_INVALID_ARG;
  if (plan_bytes < batched_plan_bytes(count)) return LATER_ERR_WORKSPACE;
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  for (int i = 0; i < count; ++i) {
    const auto& h = host_items[i];
    if (h.m < h.n || h.n < 1 || h.n > NMAX || h.lda < h.m || h.ldr < h.n || !h.A || !h.R) return LATER_ERR_INVALID_ARG;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const double ca = 2.0 * host_items[a].n * host_items[a].n * host_items[a].m;
    const double cb = 2.0 * host_items[b].n * host_items[b].n * host_items[b].m;
    return ca > cb;
  });
  std::vector<Item> items(count);
  for (int k = 0; k < count; ++k) {
    const auto& h = host_items[order[k]];
    items[k] = Item{h.A, h.R, h.lda, h.ldr, h.m, h.n, order[k], 0};
  }
  LATER_CHECK_CUDA(cudaMemcpyAsync(plan, items.data(), sizeof(Item) * count, cudaMemcpyHostToDevice, st));
  return cuda_status(cudaStreamSynchronize(st));
}

later_status_t batched_run(cudaStream_t st, int count, const void* plan, int* queue, int* status, int variant) {
  if (count < 1 || !plan || !queue) return LATER_ERR_INVALID_ARG;
  int cr, cps;
  batched_variant(variant, &cr, &cps);
  const Item* items = static_cast<const Item*>(plan);
  if (cr == 32) return launch<32>(items, count, queue, status, cps, st);
  return launch<64>(items, count, queue, status, cps, st);
}

}  // namespace later

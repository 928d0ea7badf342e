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
// CR rows (the tunable tile), so the work is throughput- not latency-bound and
// needs no inter-CTA communication. All arithmetic is FP32; reductions run in
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
    const int nq = rq / 4, total = nq * nc;
    for (int base = threadIdx.x; base < total; base += 8 * THREADS) {
      float4 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = base + u * THREADS;
        v[u] = e < total ? *reinterpret_cast<const float4*>(it.A + r0 + 4 * (e % nq) +
                                                             static_cast<int64_t>(c0 + e / nq) * it.lda)
                         : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = base + u * THREADS;
        if (e < total) *reinterpret_cast<float4*>(&dst[(e / nq) * LD + 4 * (e % nq)]) = v[u];
      }
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

// C[i][j] = sum_r Q[r][i] A[r][j] over all m rows (i < k1, j < w). Thread
// (j = t % 32, i0 = t / 32) owns C[i0 + 8u][j]; four rows per step, the Q column
// read as one float4 (the same for the whole warp: a broadcast) and the A column
// as one float4.
template <int CR>
__device__ void project(Smem<CR>& s, const Item& it, int c0, int w, int k1) {
  const int LD = CR + 4;
  const int t = threadIdx.x;
  const int j = t % PW, i0 = t / PW;  // i = i0 + 8 u
  float acc[(NMAX - PW) / 8];
#pragma unroll
  for (int u = 0; u < (NMAX - PW) / 8; ++u) acc[u] = 0.f;
  for (int r0 = 0; r0 < it.m; r0 += CR) {
    const int rows = min(CR, it.m - r0);
    __syncthreads();
    stage<CR>(s.q, it, r0, rows, 0, k1);
    stage<CR>(s.a, it, r0, rows, c0, w);
    __syncthreads();
    const int rq = (rows + 3) & ~3;
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
  __syncthreads();
#pragma unroll
  for (int u = 0; u < (NMAX - PW) / 8; ++u)
    if (i0 + 8 * u < k1) s.c[(i0 + 8 * u) * (PW + 1) + j] = (j < w) ? acc[u] : 0.f;
  __syncthreads();
}

// A_p -= Q_<p C, chunk by chunk: each thread updates a 4-row x 2-column tile of
// the staged panel chunk, reading Q as float4 along rows.
template <int CR>
__device__ void subtract(Smem<CR>& s, const Item& it, int c0, int w, int k1) {
  const int LD = CR + 4;
  const int t = threadIdx.x;
  for (int r0 = 0; r0 < it.m; r0 += CR) {
    const int rows = min(CR, it.m - r0);
    const int rq = (rows + 3) & ~3;
    __syncthreads();
    stage<CR>(s.q, it, r0, rows, 0, k1);
    stage<CR>(s.a, it, r0, rows, c0, w);
    __syncthreads();
    const int ntile = (rq / 4) * (PW / 2);
    for (int e = t; e < ntile; e += THREADS) {
      const int rt = e % (rq / 4), ct = e / (rq / 4);
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
    __syncthreads();
    for (int e = t; e < rows * w; e += THREADS) {
      const int r = e % rows, jj = e / rows;
      it.A[r0 + r + static_cast<int64_t>(c0 + jj) * it.lda] = s.a[jj * LD + r];
    }
  }
  __syncthreads();
}

// G = A_p^T A_p (w x w, into s.g): warp wp takes rows 4 wp, 4 wp + 32, ... of
// each chunk; lane (i = l / 4 .. ) owns 4 x 8 entries; warp partials are added
// in warp order.
template <int CR>
__device__ void gram(Smem<CR>& s, const Item& it, int c0, int w) {
  const int LD = CR + 4;
  const int t = threadIdx.x;
  const int lane = t % 32, wp = t / 32;
  const int ti = lane % 8, tj = lane / 8;  // entries (ti + 8 u, tj + 4 v), u < 4, v < 8
  float acc[4][8] = {};
  for (int r0 = 0; r0 < it.m; r0 += CR) {
    const int rows = min(CR, it.m - r0);
    const int rq = (rows + 3) & ~3;
    __syncthreads();
    stage<CR>(s.a, it, r0, rows, c0, w);
    __syncthreads();
    for (int r = 4 * wp; r < rq; r += 32) {
      float4 x[4], y[8];
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = *reinterpret_cast<const float4*>(&s.a[(ti + 8 * u) * LD + r]);
#pragma unroll
      for (int v = 0; v < 8; ++v) y[v] = *reinterpret_cast<const float4*>(&s.a[(tj + 4 * v) * LD + r]);
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 8; ++v)
          acc[u][v] = fmaf(x[u].w, y[v].w, fmaf(x[u].z, y[v].z, fmaf(x[u].y, y[v].y, fmaf(x[u].x, y[v].x, acc[u][v]))));
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 8; ++v) s.red[wp * PW * PW + (ti + 8 * u) * PW + tj + 4 * v] = acc[u][v];
  __syncthreads();
  for (int e = t; e < PW * PW; e += THREADS) {
    float v = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) v += s.red[q * PW * PW + e];
    const int i = e / PW, j = e % PW;
    s.g[i][j] = (i < w && j < w) ? v : 0.f;
  }
  __syncthreads();
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

// A_p <- A_p L^-T (row-wise forward substitution), one thread per row.
template <int CR>
__device__ void trsm_rows(Smem<CR>& s, const Item& it, int c0, int w) {
  for (int r = threadIdx.x; r < it.m; r += THREADS) {
    float x[PW];
#pragma unroll
    for (int j = 0; j < PW; ++j) x[j] = j < w ? it.A[r + static_cast<int64_t>(c0 + j) * it.lda] : 0.f;
#pragma unroll
    for (int j = 0; j < PW; ++j) {
      if (j < w) {
        x[j] *= s.ginv[j];
#pragma unroll
        for (int i = j + 1; i < PW; ++i)
          if (i < w) x[i] = fmaf(-x[j], s.g[i][j], x[i]);
      }
    }
#pragma unroll
    for (int j = 0; j < PW; ++j)
      if (j < w) it.A[r + static_cast<int64_t>(c0 + j) * it.lda] = x[j];
  }
  __syncthreads();
}

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
      // CGS2 against the previous panels.
      if (c0 > 0) {
        for (int pass = 0; pass < 2; ++pass) {
          project(s, it, c0, w, c0);
          for (int e = threadIdx.x; e < c0 * w; e += THREADS) {
            const int i = e % c0, j = e / c0;
            float* rp = &it.R[i + static_cast<int64_t>(c0 + j) * it.ldr];
            *rp = (pass ? *rp : 0.f) + s.c[i * (PW + 1) + j];
          }
          subtract(s, it, c0, w, c0);
        }
      }
      // CholQR2 inside the panel.
      for (int pass = 0; pass < 2; ++pass) {
        gram(s, it, c0, w);
        ok &= chol(s, w);
        trsm_rows(s, it, c0, w);
        if (pass == 0) {
          for (int e = threadIdx.x; e < PW * PW; e += THREADS) {
            const int i = e % PW, j = e / PW;  // R1 = L1^T: R1[i][j] = L1[j][i], i <= j
            r1[i][j] = (i <= j && j < w) ? s.g[j][i] : 0.f;
          }
          __syncthreads();
        }
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

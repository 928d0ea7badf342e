// Per-device status word, device properties and the elementwise kernels the
// drivers need: FP32 -> 16-bit conversion (the reference's s2h,
// util/util.cu:24-32, here vectorised and able to emit the SPLIT3 hi/lo pair),
// block copies and triangle clears (util/util.cu:172-200).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdlib>

#include "ptx.cuh"
#include "runtime.cuh"

namespace later {

__device__ int g_device_status;
// A flag that no code writes: the target of the bounded-wait self-test.
__device__ int g_never_set;

namespace {
constexpr int kMaxDev = 64;
// Per-device caches, filled on first use; two threads filling one at the same
// time store the same value.
std::atomic<int*> g_status_ptr[kMaxDev] = {};
std::atomic<int> g_nsm[kMaxDev] = {};
// A host thread may direct the status reports of the kernels it launches to a
// word of its own (the serving loop gives each request one).
thread_local int* t_status_word = nullptr;
}  // namespace

int* set_thread_status_word(int* p) {
  int* old = t_status_word;
  t_status_word = p;
  return old;
}

int* device_status_ptr() {
  if (t_status_word) return t_status_word;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return nullptr;
  int* p = g_status_ptr[dev].load(std::memory_order_acquire);
  if (!p) {
    void* q = nullptr;
    if (cudaGetSymbolAddress(&q, g_device_status) != cudaSuccess) return nullptr;
    p = static_cast<int*>(q);
    g_status_ptr[dev].store(p, std::memory_order_release);
  }
  return p;
}

int num_sms() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDev) return 148;
  int v = g_nsm[dev].load(std::memory_order_relaxed);
  if (!v) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    v = n > 0 ? n : 148;
    g_nsm[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

bool pdl_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("LATER_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

namespace {

// Each thread converts 4 consecutive rows of one column.
__global__ void convert_kernel(int m, int n, const float* __restrict__ A, int64_t lda, void* hi, void* lo,
                               int64_t ldh, int mode, int* status) {
  griddep_wait();  // inputs come from the previous kernel in the stream
  griddep_launch();
  const int col = blockIdx.y * blockDim.y + threadIdx.y;
  const int r0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
  if (col >= n || r0 >= m) return;
  const float* a = A + static_cast<int64_t>(col) * lda + r0;
  float v[4];
  const bool full = (r0 + 3 < m);
  if (full && ((reinterpret_cast<uintptr_t>(a) & 15) == 0)) {
    float4 q = *reinterpret_cast<const float4*>(a);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = (r0 + i < m) ? a[i] : 0.f;
  }
  const int64_t o = static_cast<int64_t>(col) * ldh + r0;
  if (mode == LATER_PREC_BF16) {
    __nv_bfloat16* h = reinterpret_cast<__nv_bfloat16*>(hi) + o;
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (r0 + i < m) h[i] = __float2bfloat16_rn(v[i]);
    return;
  }
  bool over = false;
  __half hv[4], lv[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    over |= fabsf(v[i]) > 65504.f;
    hv[i] = __float2half_rn(v[i]);
    lv[i] = __float2half_rn((v[i] - __half2float(hv[i])) * 2048.f);
  }
  if (over) report(status, DEV_RANGE);
  __half* h = reinterpret_cast<__half*>(hi) + o;
  __half* l = lo ? reinterpret_cast<__half*>(lo) + o : nullptr;
  if (full && ((reinterpret_cast<uintptr_t>(h) & 7) == 0) && (!l || (reinterpret_cast<uintptr_t>(l) & 7) == 0)) {
    *reinterpret_cast<uint2*>(h) = make_uint2(
        (static_cast<uint32_t>(__half_as_ushort(hv[1])) << 16) | __half_as_ushort(hv[0]),
        (static_cast<uint32_t>(__half_as_ushort(hv[3])) << 16) | __half_as_ushort(hv[2]));
    if (mode == LATER_PREC_SPLIT3 && l)
      *reinterpret_cast<uint2*>(l) = make_uint2(
          (static_cast<uint32_t>(__half_as_ushort(lv[1])) << 16) | __half_as_ushort(lv[0]),
          (static_cast<uint32_t>(__half_as_ushort(lv[3])) << 16) | __half_as_ushort(lv[2]));
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (r0 + i < m) {
        h[i] = hv[i];
        if (mode == LATER_PREC_SPLIT3 && l) l[i] = lv[i];
      }
  }
}

// Each block covers 256 rows and only visits the columns left of its last row
// (the rest of its column range lies on or above the diagonal).
__global__ void fill_strict_lower_kernel(int m, int n, float* A, int64_t lda, float v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int jend = min(n, static_cast<int>(blockIdx.x * blockDim.x + blockDim.x));
  for (int j = blockIdx.y; j < jend; j += gridDim.y)
    if (i < m && i > j) A[i + static_cast<int64_t>(j) * lda] = v;
}

__global__ void axpy2d_kernel(int m, int n, float alpha, const float* X, int64_t ldx, float* Y, int64_t ldy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (int j = blockIdx.y; j < n; j += gridDim.y)
    if (i < m) Y[i + static_cast<int64_t>(j) * ldy] += alpha * X[i + static_cast<int64_t>(j) * ldx];
}

__global__ void copy2d_kernel(int m, int n, const float* X, int64_t ldx, float* Y, int64_t ldy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (int j = blockIdx.y; j < n; j += gridDim.y)
    if (i < m) Y[i + static_cast<int64_t>(j) * ldy] = X[i + static_cast<int64_t>(j) * ldx];
}

__global__ void zero_block_kernel(int m, int n, float* X, int64_t ldx, uint16_t* xh, uint16_t* xl, int64_t ldh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  for (int j = blockIdx.y; j < n; j += gridDim.y) {
    if (X) X[i + static_cast<int64_t>(j) * ldx] = 0.f;
    if (xh) xh[i + static_cast<int64_t>(j) * ldh] = 0;
    if (xl) xl[i + static_cast<int64_t>(j) * ldh] = 0;
  }
}

}  // namespace

inline dim3 grid2d(int m, int n) {
  return dim3(static_cast<unsigned>((m + 255) / 256), static_cast<unsigned>(n < 65535 ? n : 65535));
}

later_status_t fill_strict_lower(cudaStream_t st, int m, int n, float* A, int64_t lda, float v) {
  if (m <= 0 || n <= 0) return LATER_OK;
  TraceScope trace(st, TRACE_OTHER);
  fill_strict_lower_kernel<<<dim3(static_cast<unsigned>((m + 255) / 256), static_cast<unsigned>(n < 512 ? n : 512)), 256,
                             0, st>>>(m, n, A, lda, v);
  note_launch();
  return cuda_status(cudaGetLastError());
}

later_status_t axpy2d(cudaStream_t st, int m, int n, float alpha, const float* X, int64_t ldx, float* Y,
                      int64_t ldy) {
  if (m <= 0 || n <= 0) return LATER_OK;
  TraceScope trace(st, TRACE_OTHER);
  axpy2d_kernel<<<grid2d(m, n), 256, 0, st>>>(m, n, alpha, X, ldx, Y, ldy);
  note_launch();
  return cuda_status(cudaGetLastError());
}

later_status_t copy2d(cudaStream_t st, int m, int n, const float* X, int64_t ldx, float* Y, int64_t ldy) {
  if (m <= 0 || n <= 0) return LATER_OK;
  TraceScope trace(st, TRACE_OTHER);
  copy2d_kernel<<<grid2d(m, n), 256, 0, st>>>(m, n, X, ldx, Y, ldy);
  note_launch();
  return cuda_status(cudaGetLastError());
}

later_status_t zero_block(cudaStream_t st, int m, int n, float* X, int64_t ldx, void* xh, void* xl, int64_t ldh) {
  if (m <= 0 || n <= 0) return LATER_OK;
  TraceScope trace(st, TRACE_OTHER);
  zero_block_kernel<<<grid2d(m, n), 256, 0, st>>>(m, n, X, ldx, static_cast<uint16_t*>(xh), static_cast<uint16_t*>(xl),
                                                  ldh);
  note_launch();
  return cuda_status(cudaGetLastError());
}

later_status_t convert16(cudaStream_t st, int m, int n, const float* A, int64_t lda, void* hi, void* lo,
                         int64_t ldh, int prec) {
  if (m <= 0 || n <= 0) return LATER_OK;
  if (prec == LATER_PREC_SPLIT3 && !lo) return LATER_ERR_INVALID_ARG;
  dim3 block(64, 4);
  dim3 grid(static_cast<unsigned>((m + 255) / 256), static_cast<unsigned>((n + 3) / 4));
  if (grid.y > 65535) {
    // Column counts beyond the grid limit: convert in slabs.
    for (int c = 0; c < n; c += 65535 * 4) {
      int nc = n - c < 65535 * 4 ? n - c : 65535 * 4;
      LATER_CHECK(convert16(st, m, nc, A + static_cast<int64_t>(c) * lda, lda,
                            static_cast<char*>(hi) + static_cast<int64_t>(c) * ldh * 2,
                            lo ? static_cast<char*>(lo) + static_cast<int64_t>(c) * ldh * 2 : nullptr, ldh, prec));
    }
    return LATER_OK;
  }
  TraceScope trace(st, TRACE_OTHER);
  LATER_CHECK_CUDA(
      launch_pdl(convert_kernel, grid, block, 0, st, m, n, A, lda, hi, lo, ldh, prec, device_status_ptr()));
  note_launch();
  return cuda_status(cudaGetLastError());
}


namespace {

// The two bounded waits the kernels use, each on something that never
// happens: an mbarrier phase nobody arrives on (the GEMM pipeline's wait) and
// a global flag nobody sets (the leaf's grid barrier polls a counter the same
// way). Each gives up after `budget` cycles and reports DEV_TIMEOUT.
__global__ void wait_selftest_kernel(int* status, long long budget) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  fence_barrier_init();
  if (!mbar_wait(&bar, 0, budget)) report(status, DEV_TIMEOUT);
  const long long t0 = clock64();
  while (*static_cast<volatile int*>(&g_never_set) == 0) {
    if (clock64() - t0 > budget) {
      report(status, DEV_TIMEOUT);
      break;
    }
  }
}

}  // namespace

later_status_t wait_selftest(cudaStream_t st, long long budget) {
  int* status = device_status_ptr();
  if (!status) return LATER_ERR_CUDA;
  wait_selftest_kernel<<<1, 32, 0, st>>>(status, budget > 0 ? budget : kDefaultBudgetCycles);
  note_launch();
  return cuda_status(cudaGetLastError());
}

}  // namespace later

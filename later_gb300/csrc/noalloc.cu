// Allocation-free variant of the tensor-core GEMM entry point.
//
// later_c_gemm16 takes its split-K scratch (the FP32 partial tiles summed by
// the deterministic reduction) from a caller-provided `work` buffer. Some
// callers cannot provide one: a host framework that owns every byte of device
// memory through its own pool and does not let plug-ins call the CUDA
// allocator, or a latency-critical path where cudaMalloc's implicit device
// synchronisation is not acceptable. For them, later_c_gemm16_noalloc takes
// the scratch from a fixed array in this file: a file-scope __device__ array
// that every GPU which loads the library holds until the process exits.
//
// The first call on each device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture. The array is shared by every call and
// keeps the last call's contents. Nothing in it has to start at zero: every
// partial tile is written in full before the reduction reads it. Any output
// size is accepted: the GEMM splits K only as far as the array holds the
// partial tiles (not at all when one split's tiles do not fit, which is also
// where the output alone fills the GPU). Calls whose kernels overlap on the GPU
// (different streams, or different host threads) race on the array and must
// be serialised by the caller.
#include <cuda_runtime.h>

#include <atomic>

#include "../../include/later_c.h"
#include "runtime.cuh"

namespace later {
namespace {

static __device__ __align__(256) float g_noalloc_scratch[LATER_NOALLOC_SCRATCH_FLOATS];

constexpr int kMaxDevices = 64;
std::atomic<float*> g_scratch_ptr[kMaxDevices] = {};  // filled on first use per device

// Device address of this device's scratch array (set-up on first use).
later_status_t scratch_for_current_device(float** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return LATER_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return LATER_ERR_NOT_SUPPORTED;
  float* ptr = g_scratch_ptr[dev].load(std::memory_order_acquire);
  if (!ptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return LATER_ERR_CUDA;
    ptr = static_cast<float*>(p);
    g_scratch_ptr[dev].store(ptr, std::memory_order_release);
  }
  *out = ptr;
  return LATER_OK;
}

}  // namespace
}  // namespace later

using namespace later;

extern "C" later_status_t later_c_gemm16_noalloc(later_stream_t stream, char transa, char transb, int m, int n,
                                                 int k, float alpha, const void* A, int lda, const void* B, int ldb,
                                                 float beta, const float* C, int ldc, float* D, int ldd,
                                                 int precision) {
  auto ok_t = [](char t) { return t == 'N' || t == 'n' || t == 'T' || t == 't'; };
  if (!ok_t(transa) || !ok_t(transb) || m < 0 || n < 0 || k < 1 || !A || !B || !D) return LATER_ERR_INVALID_ARG;
  if (precision != LATER_PREC_FP16 && precision != LATER_PREC_BF16) return LATER_ERR_INVALID_ARG;
  const bool an = (transa == 'N' || transa == 'n');
  const bool bn = (transb == 'N' || transb == 'n');
  if (lda < (an ? m : k) || ldb < (bn ? k : n) || ldd < m || (beta != 0.f && (!C || ldc < m)))
    return LATER_ERR_INVALID_ARG;
  float* scratch = nullptr;
  LATER_CHECK(scratch_for_current_device(&scratch));
  GemmCall g;
  g.ta = transa;
  g.tb = transb;
  g.M = m;
  g.N = n;
  g.K = k;
  g.A = Op16{A, nullptr, lda};
  g.B = Op16{B, nullptr, ldb};
  g.alpha = alpha;
  g.beta = beta;
  g.out.C = C;
  g.out.ldc = ldc;
  g.out.D = D;
  g.out.ldd = ldd;
  g.prec = precision;
  Scratch s;
  s.partial = scratch;
  s.partial_floats = LATER_NOALLOC_SCRATCH_FLOATS;
  return tc_gemm(g, s, reinterpret_cast<cudaStream_t>(stream), 0);
}

// Host-side runtime shared by the drivers: workspace arena, TMA tensor-map
// encoding, per-device properties and the internal GEMM / panel interfaces.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <utility>
#include "status.cuh"

namespace later {

// Bump allocator over caller-owned device memory. Replaces the reference's
// Mem_pool (util/mem_pool.cu:12-52), which cudaMalloc'ed its own arena and
// exit()ed on exhaustion: here the caller's `work` / `hwork` are carved up,
// and running out is a LATER_ERR_WORKSPACE status. A null base turns the
// arena into a size calculator (the *_bufsize queries run the same carving).
class Arena {
 public:
  Arena(void* base, size_t bytes) : base_(static_cast<char*>(base)), cap_(bytes) {}
  // Returns nullptr (and records the shortfall) when the request does not fit.
  template <class T>
  T* take(size_t count, size_t align = 256) {
    // Align the absolute address (the base itself may be only 16-byte aligned).
    const uintptr_t b = reinterpret_cast<uintptr_t>(base_);
    size_t off = static_cast<size_t>((b + used_ + align - 1) / align * align - b);
    size_t end = off + count * sizeof(T);
    if (end > peak_) peak_ = end;
    if (end > cap_ && base_ != nullptr) {
      failed_ = true;
      return nullptr;
    }
    used_ = end;
    return base_ ? reinterpret_cast<T*>(base_ + off) : reinterpret_cast<T*>(off + 1);
  }
  size_t used() const { return used_; }
  size_t peak() const { return peak_; }
  size_t remaining() const { return cap_ > used_ ? cap_ - used_ : 0; }
  bool failed() const { return failed_; }
  bool sizing() const { return base_ == nullptr; }
  char* cursor() const { return base_ + used_; }
  void reset(size_t to) { used_ = to; }

 private:
  char* base_;
  size_t cap_;
  size_t used_ = 0;
  size_t peak_ = 0;
  bool failed_ = false;
};

// 16-bit operand in HBM: `hi` always, `lo` only for the SPLIT3 precision.
struct Op16 {
  const void* hi = nullptr;
  const void* lo = nullptr;
  int64_t ld = 0;
};

// Output side of a tensor-core GEMM: FP32 result plus optional 16-bit copies.
struct GemmOut {
  const float* C = nullptr;  // FP32 input scaled by beta (may alias D)
  int64_t ldc = 0;
  float* D = nullptr;        // FP32 output
  int64_t ldd = 0;
  void* Dh = nullptr;        // 16-bit copy of D (hi)
  void* Dl = nullptr;        // SPLIT3 lo copy of D
  int64_t ldh = 0;
  int lower = 0;             // write only elements with row >= col + diag
  int diag = 0;
  int shadow_acc = 0;        // 16-bit copy of alpha*op(A)op(B) alone (not of D)
  int round_prod = 0;        // D = beta*C + fp32(fp16(alpha*op(A)op(B))): D holds the product's 16-bit value
};

struct GemmCall {
  char ta = 'N', tb = 'N';
  int M = 0, N = 0, K = 0;
  Op16 A, B;
  float alpha = 1.f, beta = 0.f;
  GemmOut out;
  int prec = LATER_PREC_FP16;       // operand format of A and B (SPLIT2: A hi+lo, B hi)
  int out_prec = LATER_PREC_FP16;   // format of Dh / Dl
};

struct Scratch {
  float* partial = nullptr;  // split-K partial tiles
  int64_t partial_floats = 0;
  int* counters = nullptr;   // one per output tile, zero between uses
  int n_counters = 0;
};

later_status_t tc_gemm(const GemmCall& g, const Scratch& s, cudaStream_t st, long long budget);

// Encodes a 2-D tiled map over a column-major 16-bit matrix with a 128-byte swizzle.
bool make_map16(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint64_t ld,
                uint32_t box_rows, uint32_t box_cols, bool bf16);

later_status_t convert16(cudaStream_t st, int m, int n, const float* A, int64_t lda, void* hi, void* lo,
                         int64_t ldh, int prec);

// A[i,j] = v for i > j (i < m, j < n).
later_status_t fill_strict_lower(cudaStream_t st, int m, int n, float* A, int64_t lda, float v);
// Y += alpha X  (m x n blocks).
later_status_t axpy2d(cudaStream_t st, int m, int n, float alpha, const float* X, int64_t ldx, float* Y, int64_t ldy);
// X = 0 (m x n block) and the same block of its 16-bit copies (each may be null).
later_status_t zero_block(cudaStream_t st, int m, int n, float* X, int64_t ldx, void* xh, void* xl, int64_t ldh);
// Y = X (m x n blocks).
later_status_t copy2d(cudaStream_t st, int m, int n, const float* X, int64_t ldx, float* Y, int64_t ldy);

// ------------------------------------------------------------- tracing
enum TraceKind { TRACE_GEMM = 0, TRACE_PANEL = 1, TRACE_LEAF_GEMM = 2, TRACE_OTHER = 3 };
void note_launch(int n = 1);

// Launches one kernel whose two bounded waits (an mbarrier phase and a global
// flag, neither of which ever completes) run out after `budget` cycles and
// set DEV_TIMEOUT in the device status word.
later_status_t wait_selftest(cudaStream_t st, long long budget);
// Brackets the launches issued during its lifetime with CUDA events on `st`
// while tracing is on (later_c_trace_begin); otherwise does nothing.
class TraceScope {
 public:
  TraceScope(cudaStream_t st, int kind, double flops = 0.0);
  ~TraceScope();
  TraceScope(const TraceScope&) = delete;
  TraceScope& operator=(const TraceScope&) = delete;

 private:
  cudaStream_t st_;
  int kind_;
  double flops_;
  bool on_ = false;
  cudaEvent_t a_{}, b_{};
};

inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

// Programmatic dependent launch, on unless LATER_PDL=0: the kernel may be scheduled before the previous
// kernel in `st` has ended (its prologue overlaps that kernel's tail), so it must call griddep_wait()
// (ptx.cuh) in every CTA before its first global access.
bool pdl_enabled();
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace later

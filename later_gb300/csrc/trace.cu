// Launch counting and event tracing of the library's kernels.
//
// The reference times phases with one global event pair and prints from
// inside the library (util/util.cu:4-21, Cholesky/later_rpotrf.cu:30-63). Here
// the library is silent: every kernel launch bumps a counter, and between
// later_c_trace_begin / later_c_trace_end each launch group (tensor-core GEMM,
// panel, leaf FP32 GEMM, other) is bracketed by CUDA events on its own stream,
// with the algorithmic flops of each GEMM recorded beside its device time.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "../../include/later_c.h"
#include "runtime.cuh"

namespace later {

namespace {
std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_tracing{0};
std::mutex g_mu;
struct Rec {
  cudaEvent_t a, b;
  int kind;
  double flops;
};
std::vector<Rec> g_recs;
}  // namespace

void note_launch(int n) { g_launches.fetch_add(static_cast<uint64_t>(n), std::memory_order_relaxed); }

TraceScope::TraceScope(cudaStream_t st, int kind, double flops) : st_(st), kind_(kind), flops_(flops) {
  if (!g_tracing.load(std::memory_order_relaxed)) return;
  if (cudaEventCreate(&a_) != cudaSuccess || cudaEventCreate(&b_) != cudaSuccess) return;
  cudaEventRecord(a_, st_);
  on_ = true;
}

TraceScope::~TraceScope() {
  if (!on_) return;
  cudaEventRecord(b_, st_);
  std::lock_guard<std::mutex> g(g_mu);
  g_recs.push_back(Rec{a_, b_, kind_, flops_});
}

}  // namespace later

using namespace later;

extern "C" {

uint64_t later_c_launch_count(void) { return g_launches.load(); }

void later_c_trace_begin(void) {
  std::lock_guard<std::mutex> g(g_mu);
  for (auto& r : g_recs) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  g_recs.clear();
  g_tracing.store(1);
}

later_status_t later_c_trace_end(later_trace_t* out) {
  g_tracing.store(0);
  std::lock_guard<std::mutex> g(g_mu);
  later_trace_t t{};
  later_status_t st = LATER_OK;
  for (auto& r : g_recs) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) {
      st = LATER_ERR_CUDA;
      ms = 0.f;
    }
    switch (r.kind) {
      case TRACE_GEMM:
        t.gemm_ms += ms;
        t.gemm_flops += r.flops;
        t.gemm_launches += 1;
        if (r.flops > t.top_gemm_flops) {
          t.top_gemm_flops = r.flops;
          t.top_gemm_ms = ms;
        }
        break;
      case TRACE_PANEL:
        t.panel_ms += ms;
        t.panel_launches += 1;
        break;
      case TRACE_LEAF_GEMM:
        t.leaf_gemm_ms += ms;
        t.leaf_gemm_flops += r.flops;
        t.leaf_gemm_launches += 1;
        break;
      default:
        t.other_ms += ms;
        t.other_launches += 1;
        break;
    }
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  g_recs.clear();
  if (out) *out = t;
  return st;
}

}  // extern "C"

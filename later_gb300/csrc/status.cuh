// Device-side status word and the host helpers every translation unit shares.
//
// Kernels report failures (a bounded wait that gave up, a value that overflowed
// the 16-bit operand format, a non-positive Cholesky pivot) by OR-ing a bit into
// one per-device status word. later_c_device_status() synchronises the stream,
// reads the word, clears it and maps it to a later_status_t.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "../../include/later_c.h"

namespace later {

enum : int {
  DEV_TIMEOUT = 1,   // a bounded mbarrier / flag wait ran out
  DEV_RANGE = 2,     // a value exceeded the FP16 range when written as an operand
  DEV_NUMERIC = 4,   // a non-positive pivot / zero diagonal
};

__device__ __forceinline__ void report(int* status, int bit) {
  if (status) atomicOr(status, bit);
}

// Default bound on device waits: about one second at the maximum SM clock.
constexpr long long kDefaultBudgetCycles = 2000000000LL;
// Bound used while draining operations that are already in flight.
constexpr long long kDrainBudgetCycles = 4000000000LL;

// Address of the status word the calling host thread's kernels report to: the
// thread's own word when one is set (set_thread_status_word), else this
// device's shared word (set up once per device).
int* device_status_ptr();

// Directs the status reports of the kernels this host thread launches to `p`
// (nullptr: back to the device's shared word); returns the previous setting.
int* set_thread_status_word(int* p);

struct ThreadStatusWord {
  explicit ThreadStatusWord(int* p) : old_(set_thread_status_word(p)) {}
  ~ThreadStatusWord() { set_thread_status_word(old_); }
  ThreadStatusWord(const ThreadStatusWord&) = delete;
  ThreadStatusWord& operator=(const ThreadStatusWord&) = delete;

 private:
  int* old_;
};
int num_sms();

inline later_status_t cuda_status(cudaError_t e) { return e == cudaSuccess ? LATER_OK : LATER_ERR_CUDA; }

}  // namespace later

#define LATER_CHECK_CUDA(expr)                                   \
  do {                                                           \
    cudaError_t e__ = (expr);                                    \
    if (e__ != cudaSuccess) return LATER_ERR_CUDA;               \
  } while (0)

#define LATER_CHECK(expr)                                        \
  do {                                                           \
    later_status_t s__ = (expr);                                 \
    if (s__ != LATER_OK) return s__;                             \
  } while (0)

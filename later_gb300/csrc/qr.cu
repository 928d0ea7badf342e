// Recursive Gram-Schmidt QR driver (host side).
//
// Follows the recursion of the reference's later_rgsqrf (QR/later_rgsqrf.cu:25-79):
//   [A1 | A2] = [Q1 | Q2] [R11 R12; 0 R22]
//   qr(A1);  R12 = Q1^T A2;  A2 -= Q1 R12;  qr(A2)
// with the leaf panel at n <= leaf (NMIN = 128 in the reference, :23).
// Differences, all on the GB300 side of the boundary:
//   * the 16-bit operand copy of A is kept up to date by the producers (panel
//     apply and the A2 -= Q1 R12 epilogue), so there are no s2h passes;
//   * R12 = Q1^T A2 splits K over idle SMs with a deterministic reduction;
//   * the caller's lda is honoured (the reference passes m, :70);
//   * R is written in full, zeros below the diagonal;
//   * optional CGS2 (second projection pass) and SPLIT3 / BF16 precisions;
//   * SPLIT2: R12 is one FP16 product stored at its FP16 value and A2 -= Q1 R12
//     splits Q1 into hi + lo, so the factor subtracted is the factor stored
//     (backward error at the FP32 level for 1.5x the FP16 tensor work);
//   * each leaf is one cooperative launch (leaf.cu) unless the caller asks for
//     the reference's MGS-TSQR panels.
#include <cuda_runtime.h>

#include <algorithm>

#include "householder.cuh"
#include "leaf.cuh"
#include "panel.cuh"
#include "qr.cuh"

namespace later {

Options options_from(const later_options_t* o) {
  Options r;
  if (!o) return r;
  r.prec = o->precision;
  r.cgs2 = o->cgs2 ? 1 : 0;
  r.leaf = o->leaf > 0 ? o->leaf : 128;
  r.panel = o->panel;
  r.budget = o->timeout_cycles > 0 ? o->timeout_cycles : kDefaultBudgetCycles;
  return r;
}

namespace {

constexpr int kCounters = 4096 + 64;
constexpr int kMaxHostChunks = 64;  // ints: [0,2048) panels, [2048,4096) GEMM split-K, then the fused leaf's sync

struct Ctx {
  cudaStream_t st;
  Options o;
  Arena* ws;        // float workspace (after the fixed regions)
  int* counters;    // zeroed at the start of the call
  char* sh_hi;      // 16-bit copy of A (column 0 of the full matrix)
  char* sh_lo;      // SPLIT3 lo copy
  int64_t ldh;
  void* r12h;       // 16-bit copy of the current R12 (top-level size)
  void* r12l;
  int64_t ldr12;
  float* s_tmp;     // CGS2 second-pass coefficients (top-level size)
  int64_t lds;
  int m;
  struct HostPipe* pipe = nullptr;  // host-buffer call: column chunks copied in and out around the recursion
};

inline char* col16(char* base, int64_t ld, int64_t j) { return base ? base + j * ld * 2 : nullptr; }

// Format of the 16-bit copy of Q the panels write: SPLIT2 needs Q's lo part
// (the A operand of A2 -= Q1 R12), so its panels write hi and lo as SPLIT3 does.
inline int panel_out_prec(int prec) { return prec == LATER_PREC_SPLIT2 ? LATER_PREC_SPLIT3 : prec; }
// Operand format of R12 = Q1^T A2 (SPLIT2: one FP16 product).
inline int proj_prec(int prec) { return prec == LATER_PREC_SPLIT2 ? LATER_PREC_FP16 : prec; }

Scratch gemm_scratch(Ctx& c) {
  Scratch s;
  s.counters = c.counters + 2048;
  s.n_counters = 2048;
  // Split-K partials use whatever the arena has left (never more than needed).
  const int64_t avail = static_cast<int64_t>(c.ws->remaining() / sizeof(float)) - 64;
  const int64_t cap = static_cast<int64_t>(num_sms()) * 128 * 256 * 2;
  s.partial_floats = std::max<int64_t>(0, std::min(avail, cap));
  s.partial = s.partial_floats > 0 ? reinterpret_cast<float*>(
                                         (reinterpret_cast<uintptr_t>(c.ws->cursor()) + 255) & ~uintptr_t(255))
                                   : nullptr;
  if (s.partial_floats > 0) s.partial_floats -= 64;
  return s;
}

// Host-buffer rgsqrf (later_c_rgsqrf_host): A arrives from host memory and Q,
// R go back, in chunks of columns, on two copy streams that run beside the
// recursion. Chunk k is copied in and converted to 16 bits on the `in` stream;
// the compute stream waits for it just before the first operation that reads
// those columns (the chunk's first leaf, or the trailing update of the node
// whose right half holds it). Once the leaf that finishes the chunk's last
// column has run, its columns of Q and R are final: the `out` stream copies
// them back while the recursion goes on.
struct HostPipe {
  cudaStream_t in = nullptr, out = nullptr;
  int chunk = 0, nchunks = 0;
  cudaEvent_t ready[kMaxHostChunks];  // chunk k on the device (and converted), recorded on `in`
  cudaEvent_t done[kMaxHostChunks];   // chunk k final, recorded on the compute stream
  int waited = 0;                     // chunks [0, waited) already waited for on the compute stream
  int sent = 0;                       // chunks [0, sent) queued for copy-out
  const float* hA = nullptr;
  int64_t ldha = 0;
  float* hQ = nullptr;
  int64_t ldhq = 0;
  float* hR = nullptr;
  int64_t ldhr = 0;
  float* A = nullptr;
  int64_t lda = 0;
  float* R = nullptr;
  int64_t ldr = 0;
  int n = 0;
};

// The compute stream waits until columns [0, col_end) are on the device.
later_status_t pipe_need(Ctx& c, int64_t col_end) {
  HostPipe* p = c.pipe;
  if (!p) return LATER_OK;
  const int k_end = static_cast<int>(std::min<int64_t>(p->nchunks, (col_end + p->chunk - 1) / p->chunk));
  if (k_end > p->waited) {
    LATER_CHECK_CUDA(cudaStreamWaitEvent(c.st, p->ready[k_end - 1], 0));  // `in` is in order
    p->waited = k_end;
  }
  return LATER_OK;
}

// Columns [0, col_end) of Q and R are final: queue the completed chunks' copy-out.
later_status_t pipe_done(Ctx& c, int64_t col_end) {
  HostPipe* p = c.pipe;
  if (!p) return LATER_OK;
  const int k_end = static_cast<int>(std::min<int64_t>(p->nchunks, col_end / p->chunk +
                                                                       (col_end >= p->n ? 1 : 0)));
  for (int k = p->sent; k < k_end; ++k) {
    const int64_t c0 = static_cast<int64_t>(k) * p->chunk;
    const int64_t w = std::min<int64_t>(p->chunk, p->n - c0);
    LATER_CHECK_CUDA(cudaEventRecord(p->done[k], c.st));
    LATER_CHECK_CUDA(cudaStreamWaitEvent(p->out, p->done[k], 0));
    LATER_CHECK_CUDA(cudaMemcpy2DAsync(p->hQ + c0 * p->ldhq, p->ldhq * sizeof(float), p->A + c0 * p->lda,
                                       p->lda * sizeof(float), c.m * sizeof(float), w, cudaMemcpyDeviceToHost,
                                       p->out));
    // R's column block, rows [0, c0 + w): the part on and above the diagonal
    LATER_CHECK_CUDA(cudaMemcpy2DAsync(p->hR + c0 * p->ldhr, p->ldhr * sizeof(float), p->R + c0 * p->ldr,
                                       p->ldr * sizeof(float), (c0 + w) * sizeof(float), w, cudaMemcpyDeviceToHost,
                                       p->out));
  }
  if (k_end > p->sent) p->sent = k_end;
  return LATER_OK;
}

later_status_t leaf_qr(Ctx& c, int w, float* A, int64_t lda, float* R, int64_t ldr, int64_t col) {
  if (w <= 32) {
    return tsqr_panel(c.st, c.m, A, lda, R, ldr, col16(c.sh_hi, c.ldh, col), col16(c.sh_lo, c.ldh, col), c.ldh,
                      panel_out_prec(c.o.prec), *c.ws, c.counters, c.o.budget, w);
  }
  const int w1 = split_half(w), w2 = w - w1;
  LATER_CHECK(leaf_qr(c, w1, A, lda, R, ldr, col));
  float* A2 = A + w1 * lda;
  float* R12 = R + w1 * ldr;
  LATER_CHECK(simt_tn(c.st, c.m, w1, w2, A, lda, A2, lda, R12, ldr, 0, *c.ws));
  LATER_CHECK(simt_nn_sub(c.st, c.m, w1, w2, A, lda, R12, ldr, A2, lda));
  if (c.o.cgs2) {
    LATER_CHECK(simt_tn(c.st, c.m, w1, w2, A, lda, A2, lda, c.s_tmp, c.lds, 0, *c.ws));
    LATER_CHECK(simt_nn_sub(c.st, c.m, w1, w2, A, lda, c.s_tmp, c.lds, A2, lda));
    LATER_CHECK(axpy2d(c.st, w1, w2, 1.f, c.s_tmp, c.lds, R12, ldr));
  }
  return leaf_qr(c, w2, A2, lda, R + w1 + w1 * ldr, ldr, col + w1);
}

// A leaf: one fused launch (leaf.cu) unless the caller asked for the
// reference's panel algorithm or the device / workspace cannot run it.
later_status_t leaf_top(Ctx& c, int w, float* A, int64_t lda, float* R, int64_t ldr, int64_t col) {
  LATER_CHECK(pipe_need(c, col + w));
  if ((c.o.panel == 0 || c.o.panel == 2) && w <= kLeafMaxWidth) {
    const later_status_t s =
        leaf_fused(c.st, c.m, w, A, lda, R, ldr, col16(c.sh_hi, c.ldh, col), col16(c.sh_lo, c.ldh, col), c.ldh,
                   panel_out_prec(c.o.prec), c.o.cgs2, c.o.panel == 2, *c.ws, c.counters + 4096, c.counters,
                   c.o.budget, nullptr);
    if (s != LATER_ERR_NOT_SUPPORTED && s != LATER_ERR_WORKSPACE) {
      LATER_CHECK(s);
      return pipe_done(c, col + w);
    }
  }
  LATER_CHECK(leaf_qr(c, w, A, lda, R, ldr, col));
  return pipe_done(c, col + w);
}

later_status_t rec_qr(Ctx& c, int n, float* A, int64_t lda, float* R, int64_t ldr, int64_t col) {
  if (n <= c.o.leaf) return leaf_top(c, n, A, lda, R, ldr, col);
  const int n1 = split_half(n), n2 = n - n1;
  LATER_CHECK(rec_qr(c, n1, A, lda, R, ldr, col));
  float* A2 = A + n1 * lda;
  float* R12 = R + n1 * ldr;
  Op16 Q1{col16(c.sh_hi, c.ldh, col), col16(c.sh_lo, c.ldh, col), c.ldh};
  Op16 A2h{col16(c.sh_hi, c.ldh, col + n1), col16(c.sh_lo, c.ldh, col + n1), c.ldh};
  Op16 R12h{c.r12h, c.r12l, c.ldr12};
  LATER_CHECK(pipe_need(c, col + n));  // the update reads all of A2
  const int passes = c.o.cgs2 ? 2 : 1;
  for (int pass = 0; pass < passes; ++pass) {
    // R12 (+)= Q1^T A2, FP32 into R, 16-bit copy of this pass's product. In
    // SPLIT2 the product is one FP16 GEMM and R keeps its FP16-rounded value,
    // the exact factor the update below subtracts.
    GemmCall tn;
    tn.ta = 'T';
    tn.tb = 'N';
    tn.M = n1;
    tn.N = n2;
    tn.K = c.m;
    tn.A = Q1;
    tn.B = A2h;
    tn.alpha = 1.f;
    tn.beta = pass ? 1.f : 0.f;
    tn.out.C = R12;
    tn.out.ldc = ldr;
    tn.out.D = R12;
    tn.out.ldd = ldr;
    tn.out.Dh = c.r12h;
    tn.out.Dl = c.r12l;
    tn.out.ldh = c.ldr12;
    tn.out.shadow_acc = 1;
    tn.out.round_prod = c.o.prec == LATER_PREC_SPLIT2 ? 1 : 0;
    tn.prec = proj_prec(c.o.prec);
    tn.out_prec = proj_prec(c.o.prec);
    LATER_CHECK(tc_gemm(tn, gemm_scratch(c), c.st, c.o.budget));
    // A2 -= Q1 R12 in FP32, refreshing A2's 16-bit copy (SPLIT2: Q1 = hi + lo,
    // R12 FP16; A2's copy hi only, its lo is written by A2's own panels).
    GemmCall nn;
    nn.ta = 'N';
    nn.tb = 'N';
    nn.M = c.m;
    nn.N = n2;
    nn.K = n1;
    nn.A = Q1;
    nn.B = R12h;
    nn.alpha = -1.f;
    nn.beta = 1.f;
    nn.out.C = A2;
    nn.out.ldc = lda;
    nn.out.D = A2;
    nn.out.ldd = lda;
    nn.out.Dh = const_cast<void*>(A2h.hi);
    nn.out.Dl = const_cast<void*>(A2h.lo);
    nn.out.ldh = c.ldh;
    nn.prec = c.o.prec;
    nn.out_prec = proj_prec(c.o.prec);
    LATER_CHECK(tc_gemm(nn, gemm_scratch(c), c.st, c.o.budget));
  }
  return rec_qr(c, n2, A2, lda, R + n1 + n1 * ldr, ldr, col + n1);
}

// Width of the first leaf the recursion reaches (its columns need no initial
// 16-bit copy: the panel writes it).
int first_leaf(int n, int leaf) {
  while (n > leaf) n = split_half(n);
  return n;
}

// Carves the fixed regions out of `work` (or sizes them when work is null).
// Everything after them is shared, in stream order, by the panel tree stacks,
// the leaf projection partials and the split-K partial tiles.
struct Layout {
  int* counters;
  void* r12h;
  void* r12l;
  int64_t ldr12;
  float* s_tmp;
  int64_t lds;
};

bool carve(Arena& ws, int n, const Options& o, Layout* L) {
  L->counters = ws.take<int>(kCounters);
  const int n1 = n > o.leaf ? split_half(n) : 0;
  const int n2 = n - n1;
  const bool split3 = o.prec == LATER_PREC_SPLIT3;
  L->ldr12 = round_up(std::max(n1, 8), 8);
  L->r12h = n1 ? ws.take<uint16_t>(L->ldr12 * n2) : nullptr;
  L->r12l = (n1 && split3) ? ws.take<uint16_t>(L->ldr12 * n2) : nullptr;
  L->lds = 64;
  L->s_tmp = o.cgs2 ? ws.take<float>(64 * 64) : nullptr;
  return !ws.failed();
}

}  // namespace

QrNeed rgsqrf_need(int m, int n, const Options& o) {
  QrNeed q;
  Arena a(nullptr, 0);
  Layout L;
  carve(a, n, o, &L);
  const int64_t fixed = static_cast<int64_t>(a.peak() / sizeof(float)) + 64;
  TsqrPlan plan{};
  int ncnt;
  int64_t stack;
  tsqr_plan_sizes(m, &plan, &stack, &ncnt);
  stack += 64 * kMaxTsqrLevels;
  const int64_t leaf_parts = ((m + 127) / 128) * 4096 + 128;
  const int64_t splitk = static_cast<int64_t>(num_sms()) * 128 * 256 * 2 + 128;
  q.min_work = fixed + std::max<int64_t>(stack, 4096 + 128);
  q.rec_work = fixed + std::max(std::max(std::max(stack, leaf_parts), splitk), leaf_fused_work(m));
  const int64_t ldh = round_up(m, 8);
  q.hwork = ldh * n * (o.prec == LATER_PREC_SPLIT3 || o.prec == LATER_PREC_SPLIT2 ? 2 : 1);
  return q;
}

namespace {

// Copy streams and events of the host-buffer variant, one set per host thread
// and device, created on first use and kept until exit.
struct PipeRes {
  bool ready = false;
  cudaStream_t in = nullptr, out = nullptr;
  cudaEvent_t ready_ev[kMaxHostChunks], done_ev[kMaxHostChunks], start = nullptr, end = nullptr;
};

later_status_t pipe_resources(PipeRes** out) {
  static thread_local PipeRes res[16];
  int dev = 0;
  LATER_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 16) return LATER_ERR_NOT_SUPPORTED;
  PipeRes& r = res[dev];
  if (!r.ready) {
    LATER_CHECK_CUDA(cudaStreamCreateWithFlags(&r.in, cudaStreamNonBlocking));
    LATER_CHECK_CUDA(cudaStreamCreateWithFlags(&r.out, cudaStreamNonBlocking));
    for (int k = 0; k < kMaxHostChunks; ++k) {
      LATER_CHECK_CUDA(cudaEventCreateWithFlags(&r.ready_ev[k], cudaEventDisableTiming));
      LATER_CHECK_CUDA(cudaEventCreateWithFlags(&r.done_ev[k], cudaEventDisableTiming));
    }
    LATER_CHECK_CUDA(cudaEventCreateWithFlags(&r.start, cudaEventDisableTiming));
    LATER_CHECK_CUDA(cudaEventCreateWithFlags(&r.end, cudaEventDisableTiming));
    r.ready = true;
  }
  *out = &r;
  return LATER_OK;
}

later_status_t rgsqrf_impl(cudaStream_t st, int m, int n, float* A, int64_t lda, float* R, int64_t ldr, float* work,
                           int64_t lwork, void* hwork, int64_t lhwork, const Options& o, HostPipe* pipe);

}  // namespace

later_status_t rgsqrf(cudaStream_t st, int m, int n, float* A, int64_t lda, float* R, int64_t ldr, float* work,
                      int64_t lwork, void* hwork, int64_t lhwork, const Options& o) {
  return rgsqrf_impl(st, m, n, A, lda, R, ldr, work, lwork, hwork, lhwork, o, nullptr);
}

later_status_t rgsqrf_host(cudaStream_t st, int m, int n, const float* hA, int64_t ldha, float* hQ, int64_t ldhq,
                           float* hR, int64_t ldhr, float* A, int64_t lda, float* R, int64_t ldr, float* work,
                           int64_t lwork, void* hwork, int64_t lhwork, const Options& o) {
  if (!hA || !hQ || !hR || ldha < m || ldhq < m || ldhr < n) return LATER_ERR_INVALID_ARG;
  PipeRes* res = nullptr;
  LATER_CHECK(pipe_resources(&res));
  HostPipe p;
  p.in = res->in;
  p.out = res->out;
  const int units = (n + o.leaf - 1) / std::max(o.leaf, 1);
  const int per = (units + kMaxHostChunks - 1) / kMaxHostChunks;  // leaves per chunk
  p.chunk = std::max(1, per) * o.leaf;
  p.nchunks = (n + p.chunk - 1) / p.chunk;
  for (int k = 0; k < p.nchunks; ++k) {
    p.ready[k] = res->ready_ev[k];
    p.done[k] = res->done_ev[k];
  }
  p.hA = hA;
  p.ldha = ldha;
  p.hQ = hQ;
  p.ldhq = ldhq;
  p.hR = hR;
  p.ldhr = ldhr;
  p.A = A;
  p.lda = lda;
  p.R = R;
  p.ldr = ldr;
  p.n = n;
  // the copy streams start after the caller's earlier work on `st`
  LATER_CHECK_CUDA(cudaEventRecord(res->start, st));
  LATER_CHECK_CUDA(cudaStreamWaitEvent(p.in, res->start, 0));
  LATER_CHECK_CUDA(cudaStreamWaitEvent(p.out, res->start, 0));
  const later_status_t s = rgsqrf_impl(st, m, n, A, lda, R, ldr, work, lwork, hwork, lhwork, o, &p);
  // `st` completes only after the last copy-out (also on failure: nothing may still write the caller's buffers)
  LATER_CHECK_CUDA(cudaEventRecord(res->end, p.out));
  LATER_CHECK_CUDA(cudaStreamWaitEvent(st, res->end, 0));
  LATER_CHECK_CUDA(cudaEventRecord(res->end, p.in));
  LATER_CHECK_CUDA(cudaStreamWaitEvent(st, res->end, 0));
  return s;
}

namespace {

later_status_t rgsqrf_impl(cudaStream_t st, int m, int n, float* A, int64_t lda, float* R, int64_t ldr, float* work,
                           int64_t lwork, void* hwork, int64_t lhwork, const Options& o, HostPipe* pipe) {
  if (m < 1 || n < 1 || m < n || lda < m || ldr < n || !A || !R) return LATER_ERR_INVALID_ARG;
  if (o.leaf != 32 && o.leaf != 64 && o.leaf != 128) return LATER_ERR_INVALID_ARG;
  if (o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT2) return LATER_ERR_INVALID_ARG;
  const QrNeed need = rgsqrf_need(m, n, o);
  if (!work || !hwork || lwork < need.min_work || lhwork < need.hwork) return LATER_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(hwork) & 15) != 0) return LATER_ERR_INVALID_ARG;

  Arena ws(work, static_cast<size_t>(lwork) * sizeof(float));
  Layout L;
  if (!carve(ws, n, o, &L)) return LATER_ERR_WORKSPACE;
  Ctx c;
  c.st = st;
  c.o = o;
  c.m = m;
  c.ws = &ws;
  c.counters = L.counters;
  c.ldh = round_up(m, 8);
  c.sh_hi = static_cast<char*>(hwork);
  c.sh_lo = (o.prec == LATER_PREC_SPLIT3 || o.prec == LATER_PREC_SPLIT2) ? c.sh_hi + c.ldh * n * 2 : nullptr;
  c.r12h = L.r12h;
  c.r12l = L.r12l;
  c.ldr12 = L.ldr12;
  c.s_tmp = L.s_tmp;
  c.lds = L.lds;

  LATER_CHECK_CUDA(cudaMemsetAsync(L.counters, 0, kCounters * sizeof(int), st));
  LATER_CHECK(fill_strict_lower(st, n, n, R, ldr, 0.f));
  const int f = first_leaf(n, o.leaf);
  // The columns' 16-bit copy as the projections read it (SPLIT2: hi only).
  auto convert_cols = [&](cudaStream_t s, int64_t c0, int64_t c1) -> later_status_t {
    c0 = std::max<int64_t>(c0, f);
    if (c1 <= c0) return LATER_OK;
    return convert16(s, m, static_cast<int>(c1 - c0), A + c0 * lda, lda, c.sh_hi + c0 * c.ldh * 2,
                     (c.sh_lo && o.prec == LATER_PREC_SPLIT3) ? c.sh_lo + c0 * c.ldh * 2 : nullptr, c.ldh,
                     proj_prec(o.prec));
  };
  if (pipe) {
    c.pipe = pipe;
    for (int k = 0; k < pipe->nchunks; ++k) {
      const int64_t c0 = static_cast<int64_t>(k) * pipe->chunk;
      const int64_t w = std::min<int64_t>(pipe->chunk, n - c0);
      LATER_CHECK_CUDA(cudaMemcpy2DAsync(A + c0 * lda, lda * sizeof(float), pipe->hA + c0 * pipe->ldha,
                                         pipe->ldha * sizeof(float), m * sizeof(float), w, cudaMemcpyHostToDevice,
                                         pipe->in));
      LATER_CHECK(convert_cols(pipe->in, c0, c0 + w));
      LATER_CHECK_CUDA(cudaEventRecord(pipe->ready[k], pipe->in));
    }
  } else {
    LATER_CHECK(convert_cols(st, 0, n));
  }
  return rec_qr(c, n, A, lda, R, ldr, 0);
}

}  // namespace

// ======================================================================
// Recursive Householder QR (QR/later_rhouqr.cu:27-201):
//   leaf (n <= 32): TSQR -> explicit Q -> Householder reconstruction (Y, W)
//   else: qr(left); A2 <- (I - Y1 W1^T) A2; qr(bottom-right); R12 <- A2 top,
//         zero it; W2 <- W2 - W1 (Y1^T W2)   (compact-WY merge)
// GEMMs run on the tensor cores (precision option) when n/2 > 128 and
// m > 128, else in FP32 SIMT kernels — the reference's own split (:83 Sgemm
// vs GemmEx). The top n/2 rows of each merged W2 are zeroed explicitly (the
// reference leaves them as they were in the caller's W).
namespace {

struct HCtx {
  cudaStream_t st;
  Options o;
  Arena* ws;
  int* counters;
  int64_t ldh;
  char* ah;  // 16-bit copy of A (then Y), hi / lo
  char* al;
  char* wh;  // 16-bit copy of W
  char* wl;
  float* work32;  // n1 x n2 FP32 product (top-level size)
  void* workh;    // its 16-bit copy
  void* workl;
  int64_t ldwk;
  HrScratch hr;
};

inline char* at16(char* base, int64_t ld, int64_t r, int64_t c) { return base ? base + (r + c * ld) * 2 : nullptr; }

// Longest tensor-core accumulation chain of rhouqr's SPLIT3 projections (rows of K; a multiple of 8, so
// that the 16-bit row offsets stay 16-byte aligned for the tensor maps).
constexpr int kSplit3ChainRows = 1024;

// C (k1 x k2) = X^T Z over mr rows, then Z' = Z - V C, through the tensor
// cores (16-bit copies xh/zh/vh) or FP32 SIMT.
later_status_t apply_block(HCtx& c, bool tc, int mr, int k1, int k2, const float* X, int64_t ldx, const char* xh,
                           const char* xl, float* Z, int64_t ldz, char* zh, char* zl, const float* V, int64_t ldv,
                           const char* vh, const char* vl) {
  if (!tc) {
    LATER_CHECK(simt_tn(c.st, mr, k1, k2, X, ldx, Z, ldz, c.work32, c.ldwk, 0, *c.ws));
    return simt_nn_sub(c.st, mr, k1, k2, V, ldv, c.work32, c.ldwk, Z, ldz, zh, zl, c.ldh, c.o.prec);
  }
  Scratch sc;
  sc.counters = c.counters + 2048;
  sc.n_counters = 2048;
  const int64_t avail = static_cast<int64_t>(c.ws->remaining() / sizeof(float)) - 64;
  sc.partial_floats = std::max<int64_t>(0, std::min<int64_t>(avail, static_cast<int64_t>(num_sms()) * 128 * 256 * 2));
  sc.partial = sc.partial_floats > 0 ? reinterpret_cast<float*>(
                                           (reinterpret_cast<uintptr_t>(c.ws->cursor()) + 255) & ~uintptr_t(255))
                                     : nullptr;
  if (sc.partial_floats > 0) sc.partial_floats -= 64;
  // SPLIT3: X^T Z over K = mr rows is summed in chains of at most kSplit3ChainRows rows, each chain's
  // tensor-core result added to the FP32 product in the epilogue (beta = 1, round to nearest). The
  // tensor cores' FP32 accumulation over one chain of all mr rows lets rhouqr's backward error grow with m
  // (R12 is read off the updated A2, so the projection's error enters it directly); bounded chains keep it
  // at the level of short K.
  const int chain = c.o.prec == LATER_PREC_SPLIT3 ? kSplit3ChainRows : mr;
  for (int r = 0; r < mr; r += chain) {
    const int kk = std::min(chain, mr - r);
    const bool last = r + kk >= mr;
    GemmCall tn;
    tn.ta = 'T';
    tn.tb = 'N';
    tn.M = k1;
    tn.N = k2;
    tn.K = kk;
    tn.A = Op16{xh + 2 * static_cast<int64_t>(r), xl ? xl + 2 * static_cast<int64_t>(r) : nullptr, c.ldh};
    tn.B = Op16{zh + 2 * static_cast<int64_t>(r), zl ? zl + 2 * static_cast<int64_t>(r) : nullptr, c.ldh};
    if (r > 0) {
      tn.beta = 1.f;
      tn.out.C = c.work32;
      tn.out.ldc = c.ldwk;
    }
    tn.out.D = c.work32;
    tn.out.ldd = c.ldwk;
    tn.out.Dh = last ? c.workh : nullptr;
    tn.out.Dl = last ? c.workl : nullptr;
    tn.out.ldh = c.ldwk;
    tn.prec = c.o.prec;
    tn.out_prec = c.o.prec;
    LATER_CHECK(tc_gemm(tn, sc, c.st, c.o.budget));
  }
  GemmCall nn;
  nn.ta = 'N';
  nn.tb = 'N';
  nn.M = mr;
  nn.N = k2;
  nn.K = k1;
  nn.A = Op16{vh, vl, c.ldh};
  nn.B = Op16{c.workh, c.workl, c.ldwk};
  nn.alpha = -1.f;
  nn.beta = 1.f;
  nn.out.C = Z;
  nn.out.ldc = ldz;
  nn.out.D = Z;
  nn.out.ldd = ldz;
  nn.out.Dh = zh;
  nn.out.Dl = zl;
  nn.out.ldh = c.ldh;
  nn.prec = c.o.prec;
  nn.out_prec = c.o.prec;
  return tc_gemm(nn, sc, c.st, c.o.budget);
}

// Sub-problem rows [r0, r0 + mr), columns [c0, c0 + n).
later_status_t rec_hou(HCtx& c, int r0, int mr, int c0, int n, float* A0, int64_t lda, float* W0, int64_t ldw,
                       float* R0, int64_t ldr) {
  float* A = A0 + r0 + c0 * lda;
  float* W = W0 + r0 + c0 * ldw;
  float* R = R0 + c0 + c0 * ldr;
  if (n <= 32) {
    LATER_CHECK(tsqr_panel(c.st, mr, A, lda, R, ldr, nullptr, nullptr, 0, c.o.prec, *c.ws, c.counters, c.o.budget));
    return householder_reconstruct(c.st, mr, n, A, lda, W, ldw, R, ldr, at16(c.ah, c.ldh, r0, c0),
                                   at16(c.al, c.ldh, r0, c0), at16(c.wh, c.ldh, r0, c0), at16(c.wl, c.ldh, r0, c0),
                                   c.ldh, c.o.prec, c.hr);
  }
  const int n1 = split_half(n), n2 = n - n1;
  LATER_CHECK(rec_hou(c, r0, mr, c0, n1, A0, lda, W0, ldw, R0, ldr));
  const bool tc = (n1 > 128 && mr > 128);
  // A2 <- (I - Y1 W1^T) A2 : work = W1^T A2, A2 -= Y1 work
  LATER_CHECK(apply_block(c, tc, mr, n1, n2, W, ldw, at16(c.wh, c.ldh, r0, c0), at16(c.wl, c.ldh, r0, c0),
                          A + n1 * lda, lda, at16(c.ah, c.ldh, r0, c0 + n1), at16(c.al, c.ldh, r0, c0 + n1), A, lda,
                          at16(c.ah, c.ldh, r0, c0), at16(c.al, c.ldh, r0, c0)));
  LATER_CHECK(rec_hou(c, r0 + n1, mr - n1, c0 + n1, n2, A0, lda, W0, ldw, R0, ldr));
  // R12 <- top of A2; zero it (and the top of W2) so that Y2 / W2 are full-height.
  LATER_CHECK(copy2d(c.st, n1, n2, A + n1 * lda, lda, R + n1 * ldr, ldr));
  LATER_CHECK(zero_block(c.st, n1, n2, A + n1 * lda, lda, at16(c.ah, c.ldh, r0, c0 + n1),
                         at16(c.al, c.ldh, r0, c0 + n1), c.ldh));
  LATER_CHECK(zero_block(c.st, n1, n2, W + n1 * ldw, ldw, at16(c.wh, c.ldh, r0, c0 + n1),
                         at16(c.wl, c.ldh, r0, c0 + n1), c.ldh));
  // W2 <- W2 - W1 (Y1^T W2)
  return apply_block(c, tc, mr, n1, n2, A, lda, at16(c.ah, c.ldh, r0, c0), at16(c.al, c.ldh, r0, c0), W + n1 * ldw,
                     ldw, at16(c.wh, c.ldh, r0, c0 + n1), at16(c.wl, c.ldh, r0, c0 + n1), W, ldw,
                     at16(c.wh, c.ldh, r0, c0), at16(c.wl, c.ldh, r0, c0));
}

struct HLayout {
  int* counters;
  char* wh;
  char* wl;
  float* work32;
  void* workh;
  void* workl;
  int64_t ldwk;
  HrScratch hr;
};

bool carve_hou(Arena& ws, int m, int n, const Options& o, HLayout* L) {
  const int64_t ldh = round_up(m, 8);
  const bool split3 = o.prec == LATER_PREC_SPLIT3;
  L->wh = reinterpret_cast<char*>(ws.take<uint16_t>(ldh * n));
  L->wl = split3 ? reinterpret_cast<char*>(ws.take<uint16_t>(ldh * n)) : nullptr;
  L->counters = ws.take<int>(kCounters);
  const int n1 = n > 32 ? split_half(n) : 1;
  const int n2 = std::max(n - n1, 1);
  L->ldwk = round_up(n1, 8);
  L->work32 = ws.take<float>(L->ldwk * n2);
  L->workh = ws.take<uint16_t>(L->ldwk * n2);
  L->workl = split3 ? ws.take<uint16_t>(L->ldwk * n2) : nullptr;
  L->hr.U = ws.take<float>(32 * 32);
  L->hr.T = ws.take<float>(32 * 32);
  L->hr.s = ws.take<float>(32);
  return !ws.failed();
}

}  // namespace

QrNeed rhouqr_need(int m, int n, const Options& o) {
  QrNeed q;
  Arena a(nullptr, 0);
  HLayout L;
  carve_hou(a, m, n, o, &L);
  const int64_t fixed = static_cast<int64_t>(a.peak() / sizeof(float)) + 64;
  TsqrPlan plan{};
  int ncnt;
  int64_t stack;
  tsqr_plan_sizes(m, &plan, &stack, &ncnt);
  stack += 64 * kMaxTsqrLevels;
  const int64_t parts = ((m + 127) / 128) * 4096LL * 4 + 128;  // up to 128 x 128 SIMT products
  const int64_t splitk = static_cast<int64_t>(num_sms()) * 128 * 256 * 2 + 128;
  q.min_work = fixed + std::max<int64_t>(stack, 4 * 4096 + 128);
  q.rec_work = fixed + std::max(std::max(stack, parts), splitk);
  q.hwork = round_up(m, 8) * n * (o.prec == LATER_PREC_SPLIT3 ? 2 : 1);
  return q;
}

later_status_t rhouqr(cudaStream_t st, int m, int n, float* A, int64_t lda, float* W, int64_t ldw, float* R,
                      int64_t ldr, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o) {
  if (m < 1 || n < 1 || m < n || lda < m || ldw < m || ldr < n || !A || !W || !R) return LATER_ERR_INVALID_ARG;
  if (n % 32 != 0) return LATER_ERR_INVALID_ARG;
  if (o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT3) return LATER_ERR_INVALID_ARG;
  const QrNeed need = rhouqr_need(m, n, o);
  if (!work || !hwork || lwork < need.min_work || lhwork < need.hwork) return LATER_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(hwork) & 15) != 0) return LATER_ERR_INVALID_ARG;
  Arena ws(work, static_cast<size_t>(lwork) * sizeof(float));
  HLayout L;
  if (!carve_hou(ws, m, n, o, &L)) return LATER_ERR_WORKSPACE;
  HCtx c;
  c.st = st;
  c.o = o;
  c.ws = &ws;
  c.counters = L.counters;
  c.ldh = round_up(m, 8);
  c.ah = static_cast<char*>(hwork);
  c.al = o.prec == LATER_PREC_SPLIT3 ? c.ah + c.ldh * n * 2 : nullptr;
  c.wh = L.wh;
  c.wl = L.wl;
  c.work32 = L.work32;
  c.workh = L.workh;
  c.workl = L.workl;
  c.ldwk = L.ldwk;
  c.hr = L.hr;
  LATER_CHECK_CUDA(cudaMemsetAsync(L.counters, 0, kCounters * sizeof(int), st));
  LATER_CHECK(fill_strict_lower(st, n, n, R, ldr, 0.f));
  // 16-bit copy of the columns a tensor-core update will read before any
  // kernel has rewritten them (all but the first leaf).
  const int f = n > 32 ? first_leaf(n, 32) : n;
  LATER_CHECK(convert16(st, m, n - f, A + static_cast<int64_t>(f) * lda, lda, c.ah + f * c.ldh * 2,
                        c.al ? c.al + f * c.ldh * 2 : nullptr, c.ldh, o.prec));
  return rec_hou(c, 0, m, 0, n, A, lda, W, ldw, R, ldr);
}

later_status_t ormqr(cudaStream_t st, int m, int n, float* W, int64_t ldw, const float* Y, int64_t ldy, float* work,
                     int64_t lwork) {
  if (m < 1 || n < 1 || m < n || ldw < m || ldy < m || !W || !Y) return LATER_ERR_INVALID_ARG;
  if (!work || lwork < static_cast<int64_t>(m) * n) return LATER_ERR_WORKSPACE;
  LATER_CHECK(form_q(st, m, n, W, ldw, Y, ldy, work, m));
  return copy2d(st, m, n, work, m, W, ldw);
}


// ======================================================================
// Blocked Householder QR (QR/later_bhouqr.cu:88-189): for each block of
// nb = 128 columns starting at column i,
//   panel:   rhouqr of A[i:, i:i+nb] -> Y_i (in A), local W_i, R_ii
//   update:  T = W_i^T A2, A2 -= Y_i T       (A2 = A[i:, i+nb:])
//            R[i:i+nb, i+nb:] <- A2's top rows, zeroed in A
//   merge:   W_i -= W[:, :i] (Y[:, :i]^T W_i)  (so that Q = I - W Y^T overall)
// The reference runs the update and the merge as FP32 SGEMMs; here they are
// tensor-core GEMMs in the requested precision (SPLIT3 = hi + lo operands,
// three products, FP32-level accuracy; the C++ drop-in uses it). Each GEMM
// reads 16-bit copies kept by their producers: the update's epilogue writes
// A2's copy, the merge's epilogue writes W_i's; Y_i's and the local W_i's are
// converted once after the panel. W_i's rows above i are zeroed before the
// merge (the reference leaves them as the caller's memory held them).
namespace {

constexpr int kBlockNb = 128;  // QR/later_bhouqr.cu:12 NMIN

struct BLayout {
  int* counters;
  float* T;    // nb x n   (W_i^T A2)
  float* T2;   // n x nb   (Y[:, :i]^T W_i)
  int64_t ldt, ldt2;
  char* th;    // 16-bit copies of T / T2 (hi, lo)
  char* tl;
  char* t2h;
  char* t2l;
  char* ah;    // 16-bit copy of A (Y columns left of the panel, A2 right of it)
  char* al;
  char* wh;    // 16-bit copy of W
  char* wl;
  int64_t ldh;
  float* sub_work;  // the panel's rhouqr workspace
  int64_t sub_lwork;
  void* sub_hwork;
  int64_t sub_lhwork;
};

Options panel_options(const Options& o) {
  Options p = o;
  p.prec = LATER_PREC_FP16;  // a 128-column panel's own updates run in FP32 (n/2 <= 128, :83)
  return p;
}

bool carve_bhou(Arena& fw, Arena& hw, int m, int n, const Options& o, BLayout* L) {
  const bool split3 = o.prec == LATER_PREC_SPLIT3;
  const QrNeed sub = rhouqr_need(m, std::min(n, kBlockNb), panel_options(o));
  L->counters = fw.take<int>(kCounters);
  L->ldt = round_up(kBlockNb, 8);
  L->ldt2 = round_up(n, 8);
  L->T = fw.take<float>(L->ldt * n);
  L->T2 = fw.take<float>(L->ldt2 * kBlockNb);
  L->sub_lwork = sub.rec_work;
  L->sub_work = fw.take<float>(sub.rec_work);
  L->ldh = round_up(m, 8);
  L->ah = reinterpret_cast<char*>(hw.take<uint16_t>(L->ldh * n));
  L->al = split3 ? reinterpret_cast<char*>(hw.take<uint16_t>(L->ldh * n)) : nullptr;
  L->wh = reinterpret_cast<char*>(hw.take<uint16_t>(L->ldh * n));
  L->wl = split3 ? reinterpret_cast<char*>(hw.take<uint16_t>(L->ldh * n)) : nullptr;
  L->th = reinterpret_cast<char*>(hw.take<uint16_t>(L->ldt * n));
  L->tl = split3 ? reinterpret_cast<char*>(hw.take<uint16_t>(L->ldt * n)) : nullptr;
  L->t2h = reinterpret_cast<char*>(hw.take<uint16_t>(L->ldt2 * kBlockNb));
  L->t2l = split3 ? reinterpret_cast<char*>(hw.take<uint16_t>(L->ldt2 * kBlockNb)) : nullptr;
  L->sub_lhwork = sub.hwork;
  L->sub_hwork = hw.take<uint16_t>(sub.hwork);
  return !fw.failed() && !hw.failed();
}

// D (M x N) = alpha op(A) B + beta C through the tensor cores, FP32 out plus
// its 16-bit copy (dh / dl).
later_status_t bh_gemm(cudaStream_t st, const Options& o, int* counters, Arena& fw, char ta, int M, int N, int K,
                       float alpha, const char* ah, const char* al, int64_t lda16, const char* bh, const char* bl,
                       int64_t ldb16, float beta, float* D, int64_t ldd, char* dh, char* dl, int64_t ldh16) {
  Scratch sc;
  sc.counters = counters + 2048;
  sc.n_counters = 2048;
  const int64_t avail = static_cast<int64_t>(fw.remaining() / sizeof(float)) - 64;
  sc.partial_floats = std::max<int64_t>(0, std::min<int64_t>(avail, static_cast<int64_t>(num_sms()) * 128 * 256 * 2));
  sc.partial = sc.partial_floats > 0 ? reinterpret_cast<float*>(
                                           (reinterpret_cast<uintptr_t>(fw.cursor()) + 255) & ~uintptr_t(255))
                                     : nullptr;
  if (sc.partial_floats > 0) sc.partial_floats -= 64;
  GemmCall g;
  g.ta = ta;
  g.tb = 'N';
  g.M = M;
  g.N = N;
  g.K = K;
  g.A = Op16{ah, al, lda16};
  g.B = Op16{bh, bl, ldb16};
  g.alpha = alpha;
  g.beta = beta;
  g.out.C = D;
  g.out.ldc = ldd;
  g.out.D = D;
  g.out.ldd = ldd;
  g.out.Dh = dh;
  g.out.Dl = dl;
  g.out.ldh = ldh16;
  g.prec = o.prec;
  g.out_prec = o.prec;
  return tc_gemm(g, sc, st, o.budget);
}

}  // namespace

QrNeed bhouqr_need(int m, int n, const Options& o) {
  Arena fw(nullptr, 0), hw(nullptr, 0);
  BLayout L;
  carve_bhou(fw, hw, m, n, o, &L);
  QrNeed q;
  const int64_t splitk = static_cast<int64_t>(num_sms()) * 128 * 256 * 2 + 128;
  q.min_work = static_cast<int64_t>(fw.peak() / sizeof(float)) + 64;
  q.rec_work = q.min_work + splitk;
  q.hwork = static_cast<int64_t>(hw.peak() / 2) + 128;
  return q;
}

later_status_t bhouqr(cudaStream_t st, int m, int n, float* A, int64_t lda, float* W, int64_t ldw, float* R,
                      int64_t ldr, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o) {
  if (m < 1 || n < 1 || m < n || lda < m || ldw < m || ldr < n || !A || !W || !R) return LATER_ERR_INVALID_ARG;
  if (n % 32 != 0) return LATER_ERR_INVALID_ARG;
  if (o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT3) return LATER_ERR_INVALID_ARG;
  const QrNeed need = bhouqr_need(m, n, o);
  if (!work || !hwork || lwork < need.min_work || lhwork < need.hwork) return LATER_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(hwork) & 15) != 0) return LATER_ERR_INVALID_ARG;
  Arena fw(work, static_cast<size_t>(lwork) * sizeof(float));
  Arena hw(hwork, static_cast<size_t>(lhwork) * 2);
  BLayout L;
  if (!carve_bhou(fw, hw, m, n, o, &L)) return LATER_ERR_WORKSPACE;
  const int64_t ldh = L.ldh;
  auto at = [ldh](char* base, int64_t r, int64_t c) { return base ? base + (r + c * ldh) * 2 : nullptr; };
  const Options po = panel_options(o);
  LATER_CHECK_CUDA(cudaMemsetAsync(L.counters, 0, kCounters * sizeof(int), st));
  LATER_CHECK(fill_strict_lower(st, n, n, R, ldr, 0.f));
  // A2's 16-bit copy for the first update (later ones are written by the update's epilogue).
  if (n > kBlockNb)
    LATER_CHECK(convert16(st, m, n - kBlockNb, A + kBlockNb * lda, lda, at(L.ah, 0, kBlockNb),
                          at(L.al, 0, kBlockNb), ldh, o.prec));
  for (int i = 0; i < n; i += kBlockNb) {
    const int nb = std::min(kBlockNb, n - i), mr = m - i, rest = n - i - nb;
    float* Ai = A + i + static_cast<int64_t>(i) * lda;
    float* Wi = W + static_cast<int64_t>(i) * ldw;  // column block i, from row 0
    LATER_CHECK(rhouqr(st, mr, nb, Ai, lda, Wi + i, ldw, R + i + static_cast<int64_t>(i) * ldr, ldr, L.sub_work,
                       L.sub_lwork, L.sub_hwork, L.sub_lhwork, po));
    // 16-bit copies of Y_i and the local W_i, zero above row i (so are W_i's FP32 rows)
    LATER_CHECK(convert16(st, mr, nb, Ai, lda, at(L.ah, i, i), at(L.al, i, i), ldh, o.prec));
    LATER_CHECK(convert16(st, mr, nb, Wi + i, ldw, at(L.wh, i, i), at(L.wl, i, i), ldh, o.prec));
    if (i > 0) {
      LATER_CHECK(zero_block(st, i, nb, nullptr, 0, at(L.ah, 0, i), at(L.al, 0, i), ldh));
      LATER_CHECK(zero_block(st, i, nb, Wi, ldw, at(L.wh, 0, i), at(L.wl, 0, i), ldh));
    }
    if (rest > 0) {
      float* A2 = A + i + static_cast<int64_t>(i + nb) * lda;
      // T = W_i^T A2   (nb x rest, K = mr)
      LATER_CHECK(bh_gemm(st, o, L.counters, fw, 'T', nb, rest, mr, 1.f, at(L.wh, i, i), at(L.wl, i, i), ldh,
                          at(L.ah, i, i + nb), at(L.al, i, i + nb), ldh, 0.f, L.T, L.ldt, L.th, L.tl, L.ldt));
      // A2 -= Y_i T   (mr x rest, K = nb), refreshing A2's 16-bit copy
      LATER_CHECK(bh_gemm(st, o, L.counters, fw, 'N', mr, rest, nb, -1.f, at(L.ah, i, i), at(L.al, i, i), ldh, L.th,
                          L.tl, L.ldt, 1.f, A2, lda, at(L.ah, i, i + nb), at(L.al, i, i + nb), ldh));
      LATER_CHECK(copy2d(st, nb, rest, A2, lda, R + i + static_cast<int64_t>(i + nb) * ldr, ldr));
      LATER_CHECK(zero_block(st, nb, rest, A2, lda, at(L.ah, i, i + nb), at(L.al, i, i + nb), ldh));
    }
    if (i > 0) {
      // T2 = Y[:, :i]^T W_i   (i x nb, K = m)
      LATER_CHECK(bh_gemm(st, o, L.counters, fw, 'T', i, nb, m, 1.f, L.ah, L.al, ldh, at(L.wh, 0, i),
                          at(L.wl, 0, i), ldh, 0.f, L.T2, L.ldt2, L.t2h, L.t2l, L.ldt2));
      // W_i -= W[:, :i] T2   (m x nb, K = i), refreshing W_i's 16-bit copy
      LATER_CHECK(bh_gemm(st, o, L.counters, fw, 'N', m, nb, i, -1.f, L.wh, L.wl, ldh, L.t2h, L.t2l, L.ldt2, 1.f,
                          Wi, ldw, at(L.wh, 0, i), at(L.wl, 0, i), ldh));
    }
  }
  return LATER_OK;
}

}  // namespace later

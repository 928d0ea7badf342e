// Out-of-core QR: A (and the output Q, R) in host memory, factored through a
// fixed device region (QR/later_oc_qr.cu:29-121 later_oc_qr_rec / _blk with
// BLAS/later_gemm.cu:52-189 OC_gemm). The reference recurses on the column
// halves, streams the two big products through tiled host <-> device copies
// on two streams, and factors 8192-column panels in core with later_rgsqrf.
//
// Here the same factorisation is left-looking over panels of `b` columns, the
// order that moves least data when only a few panels fit: for each panel p
//   copy A_p in;  for j < p: R_jp = Q_j^T A_p;  A_p -= Q_j R_jp   (Q_j streamed in)
//   rgsqrf(A_p) in core -> Q_p, R_pp;  copy Q_p and R[:, p] out
// Q_j is fetched on a copy stream into one of two device slots and converted
// to 16 bits there, while the tensor cores run the products with the other
// slot (double buffering over the Grace-Hopper C2C link), so the copies
// overlap the arithmetic. The projections use the precision option's operand
// formats exactly as rgsqrf's trailing updates do (SPLIT2: FP16 projection
// stored at its FP16 value, hi + lo Q in the update); with CGS2 each Q_j
// projects A_p twice while it is on the device. The caller passes the device
// region; nothing is allocated.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/later_c.h"
#include "qr.cuh"
#include "runtime.cuh"

namespace later {
namespace {

inline int proj_fmt(int prec) { return prec == LATER_PREC_SPLIT2 ? LATER_PREC_FP16 : prec; }
inline bool has_lo(int prec) { return prec == LATER_PREC_SPLIT3 || prec == LATER_PREC_SPLIT2; }

struct OcLayout {
  int* counters;
  float* Ap;             // m x b panel (FP32)
  char* aph;             // its 16-bit copy (projection operand)
  char* apl;
  float* Qs[2];          // m x b slots for Q_j (FP32 as copied in)
  char* qh[2];
  char* ql[2];
  float* Rjp;            // b x b
  char* rh;
  char* rl;
  float* Rpp;            // b x b
  float* qr_work;
  int64_t qr_lwork;
  void* qr_hwork;
  int64_t qr_lhwork;
  float* splitk;
  int64_t splitk_floats;
  int64_t ldh, ldr16;
};

bool carve_oc(Arena& a, int m, int b, const Options& o, OcLayout* L) {
  const int pf = proj_fmt(o.prec);
  L->ldh = round_up(m, 8);
  L->ldr16 = round_up(b, 8);
  L->counters = a.take<int>(4096 + 64);
  L->Ap = a.take<float>(static_cast<size_t>(m) * b);
  L->aph = reinterpret_cast<char*>(a.take<uint16_t>(L->ldh * b));
  L->apl = pf == LATER_PREC_SPLIT3 ? reinterpret_cast<char*>(a.take<uint16_t>(L->ldh * b)) : nullptr;
  for (int s = 0; s < 2; ++s) {
    L->Qs[s] = a.take<float>(static_cast<size_t>(m) * b);
    L->qh[s] = reinterpret_cast<char*>(a.take<uint16_t>(L->ldh * b));
    L->ql[s] = has_lo(o.prec) ? reinterpret_cast<char*>(a.take<uint16_t>(L->ldh * b)) : nullptr;
  }
  L->Rjp = a.take<float>(static_cast<size_t>(b) * b);
  L->rh = reinterpret_cast<char*>(a.take<uint16_t>(L->ldr16 * b));
  L->rl = pf == LATER_PREC_SPLIT3 ? reinterpret_cast<char*>(a.take<uint16_t>(L->ldr16 * b)) : nullptr;
  L->Rpp = a.take<float>(static_cast<size_t>(b) * b);
  const QrNeed q = rgsqrf_need(m, b, o);
  L->qr_lwork = q.rec_work;
  L->qr_work = a.take<float>(q.rec_work);
  L->qr_lhwork = q.hwork;
  L->qr_hwork = a.take<uint16_t>(q.hwork);
  L->splitk_floats = static_cast<int64_t>(num_sms()) * 128 * 256 * 2;
  L->splitk = a.take<float>(L->splitk_floats);
  return !a.failed();
}

struct OcRes {
  bool ready = false;
  cudaStream_t copy = nullptr;
  cudaEvent_t loaded[2], freed[2], start, end;
};

later_status_t oc_resources(OcRes** out) {
  static thread_local OcRes res[16];
  int dev = 0;
  LATER_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 16) return LATER_ERR_NOT_SUPPORTED;
  OcRes& r = res[dev];
  if (!r.ready) {
    LATER_CHECK_CUDA(cudaStreamCreateWithFlags(&r.copy, cudaStreamNonBlocking));
    for (int s = 0; s < 2; ++s) {
      LATER_CHECK_CUDA(cudaEventCreateWithFlags(&r.loaded[s], cudaEventDisableTiming));
      LATER_CHECK_CUDA(cudaEventCreateWithFlags(&r.freed[s], cudaEventDisableTiming));
    }
    LATER_CHECK_CUDA(cudaEventCreateWithFlags(&r.start, cudaEventDisableTiming));
    LATER_CHECK_CUDA(cudaEventCreateWithFlags(&r.end, cudaEventDisableTiming));
    r.ready = true;
  }
  *out = &r;
  return LATER_OK;
}

}  // namespace

int64_t oc_rgsqrf_bytes(int m, int panel, const Options& o) {
  Arena a(nullptr, 0);
  OcLayout L;
  carve_oc(a, m, panel, o, &L);
  return static_cast<int64_t>(a.peak()) + 256;
}

later_status_t oc_rgsqrf(cudaStream_t st, int m, int n, float* hA, int64_t ldha, float* hR, int64_t ldhr, int panel,
                         void* dev, int64_t dev_bytes, const Options& o) {
  if (m < 1 || n < 1 || m < n || ldha < m || ldhr < n || !hA || !hR || !dev) return LATER_ERR_INVALID_ARG;
  if (o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT2) return LATER_ERR_INVALID_ARG;
  if (panel <= 0) {  // the widest multiple of 128 columns that fits the region
    panel = 128;
    while (panel * 2 <= round_up(n, 128) && oc_rgsqrf_bytes(m, panel * 2, o) <= dev_bytes) panel *= 2;
  }
  if (panel % 32 != 0) return LATER_ERR_INVALID_ARG;
  const int b = std::min(panel, static_cast<int>(round_up(n, 32)));
  if (oc_rgsqrf_bytes(m, b, o) > dev_bytes) return LATER_ERR_WORKSPACE;
  Arena a(dev, static_cast<size_t>(dev_bytes));
  OcLayout L;
  if (!carve_oc(a, m, b, o, &L)) return LATER_ERR_WORKSPACE;
  OcRes* res = nullptr;
  LATER_CHECK(oc_resources(&res));
  const int pf = proj_fmt(o.prec);
  LATER_CHECK_CUDA(cudaEventRecord(res->start, st));
  LATER_CHECK_CUDA(cudaStreamWaitEvent(res->copy, res->start, 0));
  for (int s = 0; s < 2; ++s) LATER_CHECK_CUDA(cudaEventRecord(res->freed[s], st));

  auto gemm = [&](char ta, int M, int N, int K, float alpha, Op16 A, Op16 B, float beta, float* D, int64_t ldd,
                  char* dh, char* dl, int64_t ldh16, int prec, int out_prec, int round_prod) -> later_status_t {
    Scratch sc;
    sc.counters = L.counters;
    sc.n_counters = 4096;
    sc.partial = L.splitk;
    sc.partial_floats = L.splitk_floats;
    LATER_CHECK_CUDA(cudaMemsetAsync(L.counters, 0, 4096 * sizeof(int), st));
    GemmCall g;
    g.ta = ta;
    g.tb = 'N';
    g.M = M;
    g.N = N;
    g.K = K;
    g.A = A;
    g.B = B;
    g.alpha = alpha;
    g.beta = beta;
    g.out.C = D;
    g.out.ldc = ldd;
    g.out.D = D;
    g.out.ldd = ldd;
    g.out.Dh = dh;
    g.out.Dl = dl;
    g.out.ldh = ldh16;
    g.out.shadow_acc = ta == 'T' ? 1 : 0;
    g.out.round_prod = round_prod;
    g.prec = prec;
    g.out_prec = out_prec;
    return tc_gemm(g, sc, st, o.budget);
  };

  int loads = 0;  // Q_j loads issued so far (slot = loads % 2)
  for (int p0 = 0; p0 < n; p0 += b) {
    const int bp = std::min(b, n - p0);
    LATER_CHECK_CUDA(cudaMemcpy2DAsync(L.Ap, static_cast<size_t>(m) * sizeof(float), hA + p0 * ldha,
                                       ldha * sizeof(float), m * sizeof(float), bp, cudaMemcpyHostToDevice, st));
    if (p0 > 0) {
      // Q_0 .. Q_{p-1} went back to the host on `st`: the copy stream reads them only after that
      LATER_CHECK_CUDA(cudaEventRecord(res->start, st));
      LATER_CHECK_CUDA(cudaStreamWaitEvent(res->copy, res->start, 0));
      LATER_CHECK(convert16(st, m, bp, L.Ap, m, L.aph, L.apl, L.ldh, pf));
    }
    for (int j0 = 0; j0 < p0; j0 += b) {
      const int bj = std::min(b, p0 - j0);
      const int s = loads++ % 2;
      // fetch Q_j into slot s once the products that last read that slot are done
      LATER_CHECK_CUDA(cudaStreamWaitEvent(res->copy, res->freed[s], 0));
      LATER_CHECK_CUDA(cudaMemcpy2DAsync(L.Qs[s], static_cast<size_t>(m) * sizeof(float), hA + j0 * ldha,
                                         ldha * sizeof(float), m * sizeof(float), bj, cudaMemcpyHostToDevice,
                                         res->copy));
      LATER_CHECK(convert16(res->copy, m, bj, L.Qs[s], m, L.qh[s], L.ql[s], L.ldh,
                            has_lo(o.prec) ? LATER_PREC_SPLIT3 : o.prec));
      LATER_CHECK_CUDA(cudaEventRecord(res->loaded[s], res->copy));
      LATER_CHECK_CUDA(cudaStreamWaitEvent(st, res->loaded[s], 0));
      // with CGS2 each Q_j projects A_p twice while it is on the device
      for (int pass = 0; pass < (o.cgs2 ? 2 : 1); ++pass) {
        // R_jp (+)= Q_j^T A_p (bj x bp, K = m); the 16-bit copy holds this pass's product
        LATER_CHECK(gemm('T', bj, bp, m, 1.f, Op16{L.qh[s], pf == LATER_PREC_SPLIT3 ? L.ql[s] : nullptr, L.ldh},
                         Op16{L.aph, L.apl, L.ldh}, pass ? 1.f : 0.f, L.Rjp, b, L.rh, L.rl, L.ldr16, pf, pf,
                         o.prec == LATER_PREC_SPLIT2 ? 1 : 0));
        // A_p -= Q_j (this pass's R_jp), refreshing A_p's projection operand
        LATER_CHECK(gemm('N', m, bp, bj, -1.f, Op16{L.qh[s], L.ql[s], L.ldh}, Op16{L.rh, L.rl, L.ldr16}, 1.f, L.Ap,
                         m, L.aph, L.apl, L.ldh, o.prec, pf, 0));
      }
      LATER_CHECK_CUDA(cudaEventRecord(res->freed[s], st));
      LATER_CHECK_CUDA(cudaMemcpy2DAsync(hR + j0 + p0 * ldhr, ldhr * sizeof(float), L.Rjp, b * sizeof(float),
                                         bj * sizeof(float), bp, cudaMemcpyDeviceToHost, st));
    }
    // the panel in core
    LATER_CHECK(rgsqrf(st, m, bp, L.Ap, m, L.Rpp, b, L.qr_work, L.qr_lwork, L.qr_hwork, L.qr_lhwork, o));
    LATER_CHECK_CUDA(cudaMemcpy2DAsync(hA + p0 * ldha, ldha * sizeof(float), L.Ap, static_cast<size_t>(m) *
                                       sizeof(float), m * sizeof(float), bp, cudaMemcpyDeviceToHost, st));
    LATER_CHECK_CUDA(cudaMemcpy2DAsync(hR + p0 + p0 * ldhr, ldhr * sizeof(float), L.Rpp, b * sizeof(float),
                                       bp * sizeof(float), bp, cudaMemcpyDeviceToHost, st));
    // R below the diagonal block row: zeros (rows p0 + bp .. n of these columns)
    if (p0 + bp < n) {
      LATER_CHECK_CUDA(cudaMemsetAsync(L.Rjp, 0, static_cast<size_t>(b) * b * sizeof(float), st));
      for (int r0 = p0 + bp; r0 < n; r0 += b) {
        const int br = std::min(b, n - r0);
        LATER_CHECK_CUDA(cudaMemcpy2DAsync(hR + r0 + p0 * ldhr, ldhr * sizeof(float), L.Rjp, b * sizeof(float),
                                           br * sizeof(float), bp, cudaMemcpyDeviceToHost, st));
      }
    }
  }
  LATER_CHECK_CUDA(cudaEventRecord(res->end, res->copy));
  LATER_CHECK_CUDA(cudaStreamWaitEvent(st, res->end, 0));
  return LATER_OK;
}

}  // namespace later

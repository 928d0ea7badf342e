// Symmetric to band reduction, B = Q^T A Q with bandwidth nb
// (EVD/later_sy2sb_blocked.cu:23-186 ssytrd_sy2sb, EVD/later_sy2sb_rec.cu:62-...
// later_sy2sb_rec: the same reduction with the trailing updates deferred).
//
// For each block column i = 0, nb, ..., n - 2 nb, with lm = n - i - nb:
//   panel:  rhouqr of A[i+nb:, i:i+nb] = (I - W Y^T) [R; 0]
//   band:   A[i+nb:, i:i+nb] <- [R; 0] and its transpose above the diagonal
//   update: P = A22 W;  T = W^T P;  Z = P - 1/2 Y T;  A22 -= Y Z^T + Z Y^T
//           (A22 = A[i+nb:, i+nb:], the two-sided "ZY" form of Q^T A22 Q)
// The four products run on the tensor cores in the requested precision
// (FP16 as the reference's blocked variant, SPLIT3 for the FP32 level of its
// recursive variant's SGEMMs); A22 is kept in full symmetric storage and its
// 16-bit copy is written by the last update's epilogue, so each step reads
// A22 once for P without a conversion pass. Differences from the reference:
// one matrix is updated in place (the blocked variant factors its panels from
// the input copy A while updating A_cpy, so every panel after the first is
// stale), the band's upper triangle is written too, and the reflectors
// (Y, W per block column) can be returned for the back-transformation.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/later_c.h"
#include "qr.cuh"
#include "runtime.cuh"

namespace later {
namespace {

// Panel of the band: rows [0, nb) of the lm x nb panel get R (upper, zeros
// below), rows [nb, lm) zero; the mirrored block above the diagonal gets the
// transpose. Optionally saves the reflectors Y (unit lower) first.
__global__ void band_panel_kernel(int lm, int nb, const float* __restrict__ R, int64_t ldr, float* P, int64_t ldp,
                                  float* PT, int64_t ldpt, float* Ysave, int64_t ldy) {
  const int64_t total = static_cast<int64_t>(lm) * nb;
  for (int64_t e = blockIdx.x * 256LL + threadIdx.x; e < total; e += 256LL * gridDim.x) {
    const int64_t j = e / lm, i = e - j * lm;
    if (Ysave) Ysave[i + j * ldy] = P[i + j * ldp];
    const float v = (i < nb && i <= j) ? R[i + j * ldr] : 0.f;
    P[i + j * ldp] = v;
    PT[j + i * ldpt] = v;
  }
}

struct SLayout {
  int* counters;
  float* W;      // lm x nb (ld n) local W of the panel
  float* R;      // nb x nb
  float* P;      // n x nb: P, then Z
  float* T;      // nb x nb
  char* ah;      // 16-bit copy of A (full n x n, ld ldh)
  char* al;
  char* yh;      // 16-bit copies of Y, W, P/Z, T
  char* yl;
  char* wh;
  char* wl;
  char* ph;
  char* pl;
  char* th;
  char* tl;
  int64_t ldh, ldt;
  float* sub_work;
  int64_t sub_lwork;
  void* sub_hwork;
  int64_t sub_lhwork;
};

bool carve_sy2sb(Arena& fw, Arena& hw, int n, int nb, const Options& o, SLayout* L) {
  const bool split3 = o.prec == LATER_PREC_SPLIT3;
  Options po = o;
  po.prec = LATER_PREC_FP16;  // the panel's own updates run in FP32 at nb <= 128
  const QrNeed sub = rhouqr_need(std::max(n - nb, nb), nb, po);
  L->counters = fw.take<int>(4096 + 64);
  L->W = fw.take<float>(static_cast<size_t>(n) * nb);
  L->R = fw.take<float>(static_cast<size_t>(nb) * nb);
  L->P = fw.take<float>(static_cast<size_t>(n) * nb);
  L->T = fw.take<float>(static_cast<size_t>(nb) * nb);
  L->sub_lwork = sub.rec_work;
  L->sub_work = fw.take<float>(sub.rec_work);
  L->ldh = round_up(n, 8);
  L->ldt = round_up(nb, 8);
  auto h16 = [&](int64_t count) { return reinterpret_cast<char*>(hw.take<uint16_t>(count)); };
  L->ah = h16(L->ldh * n);
  L->al = split3 ? h16(L->ldh * n) : nullptr;
  L->yh = h16(L->ldh * nb);
  L->yl = split3 ? h16(L->ldh * nb) : nullptr;
  L->wh = h16(L->ldh * nb);
  L->wl = split3 ? h16(L->ldh * nb) : nullptr;
  L->ph = h16(L->ldh * nb);
  L->pl = split3 ? h16(L->ldh * nb) : nullptr;
  L->th = h16(L->ldt * nb);
  L->tl = split3 ? h16(L->ldt * nb) : nullptr;
  L->sub_lhwork = sub.hwork;
  L->sub_hwork = hw.take<uint16_t>(sub.hwork);
  return !fw.failed() && !hw.failed();
}

struct Ctx16 {
  cudaStream_t st;
  Options o;
  int* counters;
  Arena* fw;
};

later_status_t gemm(Ctx16& c, char ta, char tb, int M, int N, int K, float alpha, const char* ah, const char* al,
                    int64_t lda16, const char* bh, const char* bl, int64_t ldb16, float beta, float* D, int64_t ldd,
                    char* dh, char* dl, int64_t ldh16) {
  Scratch sc;
  sc.counters = c.counters;
  sc.n_counters = 4096;
  const int64_t avail = static_cast<int64_t>(c.fw->remaining() / sizeof(float)) - 64;
  sc.partial_floats = std::max<int64_t>(0, std::min<int64_t>(avail, static_cast<int64_t>(num_sms()) * 128 * 256 * 2));
  sc.partial = sc.partial_floats > 0 ? reinterpret_cast<float*>(
                                           (reinterpret_cast<uintptr_t>(c.fw->cursor()) + 255) & ~uintptr_t(255))
                                     : nullptr;
  if (sc.partial_floats > 0) sc.partial_floats -= 64;
  GemmCall g;
  g.ta = ta;
  g.tb = tb;
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
  g.prec = c.o.prec;
  g.out_prec = c.o.prec;
  return tc_gemm(g, sc, c.st, c.o.budget);
}

}  // namespace

QrNeed sy2sb_need(int n, int nb, const Options& o) {
  Arena fw(nullptr, 0), hw(nullptr, 0);
  SLayout L;
  carve_sy2sb(fw, hw, n, nb, o, &L);
  QrNeed q;
  q.min_work = static_cast<int64_t>(fw.peak() / sizeof(float)) + 64;
  q.rec_work = q.min_work + static_cast<int64_t>(num_sms()) * 128 * 256 * 2 + 128;
  q.hwork = static_cast<int64_t>(hw.peak() / 2) + 128;
  return q;
}

later_status_t sy2sb(cudaStream_t st, int n, int nb, float* A, int64_t lda, float* Y, int64_t ldy, float* W,
                     int64_t ldw, float* work, int64_t lwork, void* hwork, int64_t lhwork, const Options& o) {
  if (n < 1 || nb < 32 || nb > 128 || nb % 32 != 0 || n % nb != 0 || lda < n || !A) return LATER_ERR_INVALID_ARG;
  if ((Y && ldy < n) || (W && ldw < n)) return LATER_ERR_INVALID_ARG;
  if (o.prec < LATER_PREC_FP16 || o.prec > LATER_PREC_SPLIT3) return LATER_ERR_INVALID_ARG;
  const QrNeed need = sy2sb_need(n, nb, o);
  if (!work || !hwork || lwork < need.min_work || lhwork < need.hwork) return LATER_ERR_WORKSPACE;
  if ((reinterpret_cast<uintptr_t>(hwork) & 15) != 0) return LATER_ERR_INVALID_ARG;
  Arena fw(work, static_cast<size_t>(lwork) * sizeof(float));
  Arena hw(hwork, static_cast<size_t>(lhwork) * 2);
  SLayout L;
  if (!carve_sy2sb(fw, hw, n, nb, o, &L)) return LATER_ERR_WORKSPACE;
  const int64_t ldh = L.ldh;
  auto at = [ldh](char* base, int64_t r, int64_t c) { return base ? base + (r + c * ldh) * 2 : nullptr; };
  Options po = o;
  po.prec = LATER_PREC_FP16;
  Ctx16 c{st, o, L.counters, &fw};
  LATER_CHECK_CUDA(cudaMemsetAsync(L.counters, 0, (4096 + 64) * sizeof(int), st));
  if (Y) LATER_CHECK_CUDA(cudaMemset2DAsync(Y, ldy * sizeof(float), 0, n * sizeof(float), n, st));
  if (W) LATER_CHECK_CUDA(cudaMemset2DAsync(W, ldw * sizeof(float), 0, n * sizeof(float), n, st));
  if (n <= nb) return LATER_OK;
  LATER_CHECK(convert16(st, n - nb, n - nb, A + nb + static_cast<int64_t>(nb) * lda, lda, at(L.ah, nb, nb),
                        at(L.al, nb, nb), ldh, o.prec));
  for (int i = 0; i + nb < n; i += nb) {
    const int lm = n - i - nb;
    const int r0 = i + nb;  // first row / column of A22
    float* Pan = A + r0 + static_cast<int64_t>(i) * lda;
    float* PanT = A + i + static_cast<int64_t>(r0) * lda;
    float* A22 = A + r0 + static_cast<int64_t>(r0) * lda;
    LATER_CHECK(rhouqr(st, lm, nb, Pan, lda, L.W, n, L.R, nb, L.sub_work, L.sub_lwork, L.sub_hwork, L.sub_lhwork,
                       po));
    // 16-bit copies of Y (the panel) and W before the panel becomes part of the band
    LATER_CHECK(convert16(st, lm, nb, Pan, lda, L.yh, L.yl, ldh, o.prec));
    LATER_CHECK(convert16(st, lm, nb, L.W, n, L.wh, L.wl, ldh, o.prec));
    if (W) LATER_CHECK(copy2d(st, lm, nb, L.W, n, W + r0 + static_cast<int64_t>(i) * ldw, ldw));
    band_panel_kernel<<<static_cast<int>(std::min<int64_t>((static_cast<int64_t>(lm) * nb + 255) / 256, 2048)), 256,
                        0, st>>>(lm, nb, L.R, nb, Pan, lda, PanT, lda,
                                 Y ? Y + r0 + static_cast<int64_t>(i) * ldy : nullptr, ldy);
    note_launch();
    LATER_CHECK_CUDA(cudaGetLastError());
    // P = A22 W   (lm x nb, K = lm)
    LATER_CHECK(gemm(c, 'N', 'N', lm, nb, lm, 1.f, at(L.ah, r0, r0), at(L.al, r0, r0), ldh, L.wh, L.wl, ldh, 0.f,
                     L.P, n, L.ph, L.pl, ldh));
    // T = W^T P   (nb x nb, K = lm)
    LATER_CHECK(gemm(c, 'T', 'N', nb, nb, lm, 1.f, L.wh, L.wl, ldh, L.ph, L.pl, ldh, 0.f, L.T, nb, L.th, L.tl,
                     L.ldt));
    // Z = P - 1/2 Y T   (in place over P, K = nb)
    LATER_CHECK(gemm(c, 'N', 'N', lm, nb, nb, -0.5f, L.yh, L.yl, ldh, L.th, L.tl, L.ldt, 1.f, L.P, n, L.ph, L.pl,
                     ldh));
    // A22 -= Y Z^T + Z Y^T   (lm x lm, K = nb); the second refreshes A22's 16-bit copy
    LATER_CHECK(gemm(c, 'N', 'T', lm, lm, nb, -1.f, L.yh, L.yl, ldh, L.ph, L.pl, ldh, 1.f, A22, lda, nullptr,
                     nullptr, 0));
    LATER_CHECK(gemm(c, 'N', 'T', lm, lm, nb, -1.f, L.ph, L.pl, ldh, L.yh, L.yl, ldh, 1.f, A22, lda,
                     at(L.ah, r0, r0), at(L.al, r0, r0), ldh));
  }
  return LATER_OK;
}

}  // namespace later

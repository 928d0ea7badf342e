// A client written against LATER.h the way the reference's tests call it
// (test/test_qr.cu:66-176, test/test_potrf.cu, test/test_trsm.cu): buffers
// sized as the reference sizes them, a cudaCtxt, and no other API. Checks
// each result on the host in double precision; exit code 0 = all within bounds.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "LATER.h"

static std::vector<float> randn(size_t n, unsigned seed) {
  std::vector<float> v(n);
  unsigned s = seed;
  for (size_t i = 0; i < n; i += 2) {  // Box-Muller on a 32-bit LCG
    s = s * 1664525u + 1013904223u;
    double u1 = ((s >> 8) + 1.0) / 16777217.0;
    s = s * 1664525u + 1013904223u;
    double u2 = ((s >> 8) + 0.5) / 16777216.0;
    double r = std::sqrt(-2.0 * std::log(u1));
    v[i] = static_cast<float>(r * std::cos(6.283185307179586 * u2));
    if (i + 1 < n) v[i + 1] = static_cast<float>(r * std::sin(6.283185307179586 * u2));
  }
  return v;
}

static double qr_bwd(int m, int n, const std::vector<float>& A, const std::vector<float>& Q,
                     const std::vector<float>& R) {
  double num = 0, den = 0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0;
      for (int k = 0; k <= j; ++k) s += static_cast<double>(Q[i + (size_t)k * m]) * R[k + (size_t)j * n];
      const double d = A[i + (size_t)j * m] - s;
      num += d * d;
      den += static_cast<double>(A[i + (size_t)j * m]) * A[i + (size_t)j * m];
    }
  return std::sqrt(num / den);
}

#define CK(x)                                                   \
  do {                                                          \
    cudaError_t e = (x);                                        \
    if (e != cudaSuccess) {                                     \
      std::printf("CUDA error %s at %d\n", cudaGetErrorString(e), __LINE__); \
      return 2;                                                 \
    }                                                           \
  } while (0)

int main() {
  int fails = 0;
  const int m = 2048, n = 512;
  std::vector<float> hA = randn((size_t)m * n, 7);
  float *A, *R, *W, *work, *U;
  __half* hwork;
  CK(cudaMalloc(&A, sizeof(float) * m * n));
  CK(cudaMalloc(&R, sizeof(float) * n * n));
  CK(cudaMalloc(&W, sizeof(float) * m * n));
  CK(cudaMalloc(&work, sizeof(float) * m * n));
  CK(cudaMalloc(&hwork, sizeof(__half) * m * n));
  CK(cudaMalloc(&U, sizeof(float) * 32 * 32));
  cudaCtxt ctxt{};

  // rgsqrf with the reference test's buffer sizes (test/test_qr.cu:69-74)
  CK(cudaMemcpy(A, hA.data(), sizeof(float) * m * n, cudaMemcpyHostToDevice));
  later_rgsqrf(ctxt, m, n, A, m, R, n, work, m / 256 * 32 * n, hwork, m * n);
  CK(cudaDeviceSynchronize());
  std::vector<float> Q((size_t)m * n), hR((size_t)n * n);
  CK(cudaMemcpy(Q.data(), A, sizeof(float) * m * n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hR.data(), R, sizeof(float) * n * n, cudaMemcpyDeviceToHost));
  double e1 = qr_bwd(m, n, hA, Q, hR);
  std::printf("later_rgsqrf status %d  ||A-QR||/||A|| = %.3e\n", (int)later_get_last_status(), e1);
  fails += (later_get_last_status() != LATER_OK || !(e1 < 5e-4));

  // rhouqr + ormqr with the reference test's buffers (test/test_qr.cu:107-128)
  CK(cudaMemcpy(A, hA.data(), sizeof(float) * m * n, cudaMemcpyHostToDevice));
  later_rhouqr(ctxt, m, n, A, m, W, m, R, n, work, m * n, hwork, m * n, U);
  later_ormqr(m, n, W, m, A, m, work);
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(Q.data(), W, sizeof(float) * m * n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hR.data(), R, sizeof(float) * n * n, cudaMemcpyDeviceToHost));
  double e2 = qr_bwd(m, n, hA, Q, hR);
  std::printf("later_rhouqr+ormqr status %d  ||A-QR||/||A|| = %.3e\n", (int)later_get_last_status(), e2);
  fails += (later_get_last_status() != LATER_OK || !(e2 < 5e-4));

  // bhouqr + ormqr2 with the reference test's buffers (test/test_qr.cu:140-176, algo 3)
  CK(cudaMemcpy(A, hA.data(), sizeof(float) * m * n, cudaMemcpyHostToDevice));
  later_bhouqr(m, n, A, m, W, m, R, n, work, m * n, hwork, m * n, U);
  later_ormqr2(m, n, W, m, A, m, work);
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(Q.data(), W, sizeof(float) * m * n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(hR.data(), R, sizeof(float) * n * n, cudaMemcpyDeviceToHost));
  double e2b = qr_bwd(m, n, hA, Q, hR);
  std::printf("later_bhouqr+ormqr2 status %d  ||A-QR||/||A|| = %.3e\n", (int)later_get_last_status(), e2b);
  fails += (later_get_last_status() != LATER_OK || !(e2b < 3e-6));

  // rpotrf on the reference test's SPD input T T^T, T = tril(0.1) (test/test_potrf.cu:38-62)
  const int np = 512;
  std::vector<double> T((size_t)np * np, 0.0);
  for (int j = 0; j < np; ++j)
    for (int i = j; i < np; ++i) T[i + (size_t)j * np] = 0.1;
  std::vector<float> S((size_t)np * np);
  for (int j = 0; j < np; ++j)
    for (int i = 0; i < np; ++i) {
      double s = 0;
      for (int k = 0; k <= std::min(i, j); ++k) s += T[i + (size_t)k * np] * T[j + (size_t)k * np];
      S[i + (size_t)j * np] = static_cast<float>(s);
    }
  CK(cudaMemcpy(A, S.data(), sizeof(float) * np * np, cudaMemcpyHostToDevice));
  later_rpotrf('l', np, A, np, work, hwork);
  CK(cudaDeviceSynchronize());
  std::vector<float> L((size_t)np * np);
  CK(cudaMemcpy(L.data(), A, sizeof(float) * np * np, cudaMemcpyDeviceToHost));
  double num = 0, den = 0;
  for (int j = 0; j < np; ++j)
    for (int i = j; i < np; ++i) {
      double s = 0;
      for (int k = 0; k <= j; ++k) s += static_cast<double>(L[i + (size_t)k * np]) * L[j + (size_t)k * np];
      num += (S[i + (size_t)j * np] - s) * (S[i + (size_t)j * np] - s);
      den += static_cast<double>(S[i + (size_t)j * np]) * S[i + (size_t)j * np];
    }
  double e3 = std::sqrt(num / den);
  std::printf("later_rpotrf status %d  ||A-LL^T||/||A|| = %.3e\n", (int)later_get_last_status(), e3);
  fails += (later_get_last_status() != LATER_OK || !(e3 < 1e-5));

  // rtrsm('l','r','t') on the reference test's constant input (test/test_trsm.cu:44-66)
  const int mt = 1024, nt = 512;
  std::vector<float> Lc((size_t)nt * nt, 0.f), Bc((size_t)mt * nt);
  for (int j = 0; j < nt; ++j)
    for (int i = j; i < nt; ++i) Lc[i + (size_t)j * nt] = 0.1f;
  for (int j = 0; j < nt; ++j)
    for (int i = 0; i < mt; ++i) Bc[i + (size_t)j * mt] = 0.1f * (nt - j);  // ones * L
  float *dL, *dB;
  CK(cudaMalloc(&dL, sizeof(float) * nt * nt));
  CK(cudaMalloc(&dB, sizeof(float) * mt * nt));
  CK(cudaMemcpy(dL, Lc.data(), sizeof(float) * nt * nt, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dB, Bc.data(), sizeof(float) * mt * nt, cudaMemcpyHostToDevice));
  later_rtrsm(nullptr, 'l', 'r', 't', mt, nt, dL, nt, dB, mt, hwork);
  CK(cudaDeviceSynchronize());
  std::vector<float> X((size_t)mt * nt);
  CK(cudaMemcpy(X.data(), dB, sizeof(float) * mt * nt, cudaMemcpyDeviceToHost));
  num = den = 0;
  for (int j = 0; j < nt; ++j)
    for (int i = 0; i < mt; i += 7) {
      double s = 0;
      for (int k = 0; k <= j; ++k) s += static_cast<double>(X[i + (size_t)k * mt]) * Lc[j + (size_t)k * nt];
      num += (Bc[i + (size_t)j * mt] - s) * (Bc[i + (size_t)j * mt] - s);
      den += static_cast<double>(Bc[i + (size_t)j * mt]) * Bc[i + (size_t)j * mt];
    }
  double e4 = std::sqrt(num / den);
  std::printf("later_rtrsm status %d  ||X L^T - B||/||B|| = %.3e\n", (int)later_get_last_status(), e4);
  fails += (later_get_last_status() != LATER_OK || !(e4 < 1e-3));

  // unsupported rtrsm flags report an error instead of the reference's silent no-op
  later_rtrsm(nullptr, 'u', 'l', 'n', mt, nt, dL, nt, dB, mt, hwork);
  fails += (later_get_last_status() != LATER_ERR_NOT_SUPPORTED);

  std::printf(fails ? "FAILED (%d)\n" : "ALL OK\n", fails);
  return fails ? 1 : 0;
}

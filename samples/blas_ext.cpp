// Drop-in demo of the element-wise BLAS-1 calls, the matrix copy/transpose
// extensions and blas::_symm through include/portblas_gb.h, verified against
// host loops.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "portblas_gb.h"

static float* upload(const std::vector<float>& v) {
  float* d = nullptr;
  cudaMalloc((void**)&d, v.size() * sizeof(float));
  cudaMemcpy(d, v.data(), v.size() * sizeof(float), cudaMemcpyHostToDevice);
  return d;
}
static std::vector<float> download(const float* d, size_t n) {
  std::vector<float> v(n);
  cudaMemcpy(v.data(), d, n * sizeof(float), cudaMemcpyDeviceToHost);
  return v;
}

int main() {
  std::mt19937 gen(7);
  std::uniform_real_distribution<float> U(-2.f, 5.f);
  const int n = 1003;
  std::vector<float> x(n), y(n);
  for (auto& e : x) e = U(gen);
  for (auto& e : y) e = U(gen);
  blas::SB_Handle sb(nullptr);
  float *dx = upload(x), *dy = upload(y), *dz = upload(y);
  double err = 0;

  blas::_axpy(sb, n, 2.5f, dx, 1, dy, 1);  // y <- 2.5 x + y
  blas::_scal(sb, n, -0.5f, dy, 1);        // y <- -0.5 y
  auto ev = blas::_copy(sb, n, dy, 1, dz, 1);
  sb.wait(ev);
  auto z = download(dz, n);
  for (int i = 0; i < n; ++i) err = std::fmax(err, std::fabs(z[i] - (-0.5f * (2.5f * x[i] + y[i]))));
  double ref = 0.25;
  for (int i = 0; i < n; ++i) ref += double(x[i]) * z[i];
  float sds = blas::_sdsdot(sb, n, 0.25f, dx, 1, dz, 1);
  err = std::fmax(err, std::fabs(sds - ref) / std::fabs(ref));

  // omatcopy (transposed, scaled) and out-of-place transpose of a 70 x 33 matrix
  const int m = 70, k = 33;
  std::vector<float> A(m * k);
  for (auto& e : A) e = U(gen);
  float *dA = upload(A), *dB = upload(std::vector<float>(m * k)), *dT = upload(std::vector<float>(m * k));
  blas::extension::_omatcopy(sb, 't', m, k, 2.0f, dA, m, dB, k);
  ev = blas::extension::_transpose<float>(sb, m, k, dA, m, dT, k);
  sb.wait(ev);
  auto B = download(dB, m * k), T = download(dT, m * k);
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < m; ++i) {
      err = std::fmax(err, std::fabs(B[j + i * k] - 2.0f * A[i + j * m]));
      err = std::fmax(err, std::fabs(T[j + i * k] - A[i + j * m]));
    }

  // symm, side 'l', upper triangle of a 40 x 40 matrix, 40 x 25 B
  const int sm = 40, sn = 25;
  std::vector<float> S(sm * sm), SB(sm * sn), SC(sm * sn);
  for (auto* v : {&S, &SB, &SC})
    for (auto& e : *v) e = U(gen);
  float *dS = upload(S), *dSB = upload(SB), *dSC = upload(SC);
  ev = blas::_symm(sb, 'l', 'u', sm, sn, 1.5f, dS, sm, dSB, sm, 0.5f, dSC, sm);
  sb.wait(ev);
  auto C = download(dSC, sm * sn);
  for (int j = 0; j < sn; ++j)
    for (int i = 0; i < sm; ++i) {
      double acc = 0;
      for (int p = 0; p < sm; ++p) {
        const float a = i <= p ? S[i + p * sm] : S[p + i * sm];
        acc += double(a) * SB[p + j * sm];
      }
      const double want = 1.5 * acc + 0.5 * SC[i + j * sm];
      err = std::fmax(err, std::fabs(C[i + j * sm] - want) / (1 + std::fabs(want)));
    }

  for (float* p : {dx, dy, dz, dA, dB, dT, dS, dSB, dSC}) cudaFree(p);
  std::printf("blas_ext sample: max error %.3g\n", err);
  return err < 1e-3 ? 0 : 1;
}

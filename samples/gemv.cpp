// Drop-in demo of blas::_gemv and the BLAS-1 / reduction calls through
// include/portblas_gb.h, verified against host loops.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "portblas_gb.h"

int main() {
  const int m = 1023, n = 514, lda = m;
  std::vector<float> A(lda * n), x(n), y(m);
  std::mt19937 gen(11);
  std::uniform_real_distribution<float> U(-2.f, 5.f);
  for (auto* v : {&A, &x, &y})
    for (auto& e : *v) e = U(gen);
  blas::SB_Handle sb_handle(nullptr);
  float *dA, *dx, *dy, *dr, *dout;
  int* di;
  cudaMalloc((void**)&dA, A.size() * 4);
  cudaMalloc((void**)&dx, x.size() * 4);
  cudaMalloc((void**)&dy, y.size() * 4);
  cudaMalloc((void**)&dr, 4);
  cudaMalloc((void**)&di, 4);
  cudaMalloc((void**)&dout, n * 4);
  cudaMemcpy(dA, A.data(), A.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dx, x.data(), x.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dy, y.data(), y.size() * 4, cudaMemcpyHostToDevice);

  auto ev = blas::_gemv(sb_handle, 'n', m, n, 1.5f, dA, lda, dx, 1, 0.5f, dy, 1);
  sb_handle.wait(ev);
  std::vector<float> out(m);
  cudaMemcpy(out.data(), dy, m * 4, cudaMemcpyDeviceToHost);
  double err = 0;
  for (int i = 0; i < m; ++i) {
    double acc = 0;
    for (int j = 0; j < n; ++j) acc += double(A[i + j * lda]) * x[j];
    err = std::fmax(err, std::fabs(1.5 * acc + 0.5 * y[i] - out[i]) / (1 + std::fabs(1.5 * acc)));
  }

  // BLAS-1: sync overloads return host scalars, async ones write device memory
  double ref_asum = 0, ref_dot = 0;
  int ref_imax = 0;
  for (int j = 0; j < n; ++j) {
    ref_asum += std::fabs(x[j]);
    ref_dot += double(x[j]) * x[j];
    if (std::fabs(x[j]) > std::fabs(x[ref_imax])) ref_imax = j;
  }
  float asum = blas::_asum(sb_handle, n, dx, 1);
  float nrm2 = blas::_nrm2(sb_handle, n, dx, 1);
  float dot = blas::_dot(sb_handle, n, dx, 1, dx, 1);
  int imax = blas::_iamax(sb_handle, n, dx, 1);
  auto ev2 = blas::_iamax(sb_handle, n, dx, 1, di);
  sb_handle.wait(ev2);
  int imax_async = -1;
  cudaMemcpy(&imax_async, di, 4, cudaMemcpyDeviceToHost);

  // extension::_reduction, inner (column sums)
  auto ev3 = blas::extension::_reduction<blas::AddOperator, float>(sb_handle, dA, lda, dout, m, n,
                                                                   blas::reduction_dim_t::inner);
  sb_handle.wait(ev3);
  std::vector<float> colsum(n);
  cudaMemcpy(colsum.data(), dout, n * 4, cudaMemcpyDeviceToHost);
  double rerr = 0;
  for (int j = 0; j < n; ++j) {
    double s = 0;
    for (int i = 0; i < m; ++i) s += A[i + j * lda];
    rerr = std::fmax(rerr, std::fabs(s - colsum[j]) / (1 + std::fabs(s)));
  }
  bool ok = err < 1e-5 && std::fabs(asum - ref_asum) < 1e-4 * ref_asum &&
            std::fabs(nrm2 - std::sqrt(ref_dot)) < 1e-5 * std::sqrt(ref_dot) &&
            std::fabs(dot - ref_dot) < 1e-5 * ref_dot && imax == ref_imax && imax_async == ref_imax &&
            rerr < 1e-5;
  std::printf("gemv err %.3g asum %.6g/%.6g nrm2 %.6g dot %.6g iamax %d/%d/%d reduction err %.3g -> %s\n", err,
              asum, ref_asum, nrm2, dot, imax, imax_async, ref_imax, rerr, ok ? "OK" : "FAIL");
  cudaFree(dA);
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dr);
  cudaFree(di);
  cudaFree(dout);
  return ok ? 0 : 1;
}

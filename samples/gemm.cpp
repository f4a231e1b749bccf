// Drop-in demo: the portBLAS gemm sample's calls (samples/gemm.cpp in portBLAS)
// against the GB300 library through include/portblas_gb.h.  Verifies the
// result with a host loop and exits non-zero on mismatch.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "portblas_gb.h"

int main() {
  const int m = 257, n = 129, k = 65, lda = m, ldb = k, ldc = m;
  const float alpha = 1.5f, beta = 0.5f;
  std::vector<float> A(lda * k), B(ldb * n), C(ldc * n);
  std::mt19937 gen(7);
  std::uniform_real_distribution<float> U(-1.f, 1.f);
  for (auto* v : {&A, &B, &C})
    for (auto& x : *v) x = U(gen);

  cudaStream_t q;
  cudaStreamCreate(&q);
  blas::SB_Handle sb_handle(q);
  float *dA, *dB, *dC;
  cudaMalloc((void**)&dA, A.size() * 4);
  cudaMalloc((void**)&dB, B.size() * 4);
  cudaMalloc((void**)&dC, C.size() * 4);
  cudaMemcpy(dA, A.data(), A.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dB, B.data(), B.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dC, C.data(), C.size() * 4, cudaMemcpyHostToDevice);

  auto ev = blas::_gemm(sb_handle, 'n', 'n', m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc);
  sb_handle.wait(ev);

  std::vector<float> out(C.size());
  cudaMemcpy(out.data(), dC, out.size() * 4, cudaMemcpyDeviceToHost);
  double maxerr = 0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double acc = 0;
      for (int p = 0; p < k; ++p) acc += double(A[i + p * lda]) * double(B[p + j * ldb]);
      double ref = alpha * acc + beta * double(C[i + j * ldc]);
      maxerr = std::fmax(maxerr, std::fabs(ref - out[i + j * ldc]));
    }
  // errors surface as the same exception types as portBLAS
  bool threw = false;
  try {
    blas::_gemm(sb_handle, 'x', 'n', m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc);
  } catch (const std::invalid_argument&) {
    threw = true;
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  std::printf("gemm max abs err %.3g, invalid trans threw: %d\n", maxerr, int(threw));
  return (maxerr < 1e-4 && threw) ? 0 : 1;
}

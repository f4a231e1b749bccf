// Drop-in demo: an uneven batch of GEMMs through blas::extension::_gemm_grouped
// and a reusable blas::extension::gemm_grouped_plan (FP32 and bfloat16
// inputs), and the lifetime of the events the blas:: calls return.  Verifies
// against a host loop and exits non-zero on any mismatch.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <set>
#include <vector>

#include "portblas_gb.h"

namespace {

// bfloat16 bits of x, rounded to nearest even (finite inputs)
uint16_t to_bf16(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  u += 0x7fffu + ((u >> 16) & 1u);
  return uint16_t(u >> 16);
}
float from_bf16(uint16_t h) {
  uint32_t u = uint32_t(h) << 16;
  float x;
  std::memcpy(&x, &u, 4);
  return x;
}

struct Problem {
  int64_t m, n, k;
  char ta, tb;
  float alpha, beta;
  std::vector<float> A, B, C;  // host values (bf16-rounded for the bf16 run)
  int64_t lda, ldb, ldc;
};

template <typename in_t>
int run(cudaStream_t q, bool use_plan) {
  blas::SB_Handle sb(q);
  std::mt19937 gen(11);
  std::uniform_real_distribution<float> U(-1.f, 1.f);
  const int64_t dims[][3] = {{70, 150, 40}, {130, 33, 300}, {1, 1, 1}, {256, 200, 129}, {17, 300, 64}};
  const int count = 5;
  std::vector<Problem> P(count);
  std::vector<in_t*> dA(count), dB(count);
  std::vector<float*> dC(count);
  for (int i = 0; i < count; ++i) {
    Problem& p = P[i];
    p.m = dims[i][0], p.n = dims[i][1], p.k = dims[i][2];
    p.ta = (i % 2) ? 't' : 'n';
    p.tb = (i % 3 == 1) ? 't' : 'n';
    p.alpha = 1.0f + 0.25f * i;
    p.beta = (i % 2) ? 0.5f : 0.0f;
    p.lda = (p.ta == 'n' ? p.m : p.k) + 1;
    p.ldb = (p.tb == 'n' ? p.k : p.n) + 2;
    p.ldc = p.m + 3;
    p.A.resize(size_t(p.lda) * (p.ta == 'n' ? p.k : p.m));
    p.B.resize(size_t(p.ldb) * (p.tb == 'n' ? p.n : p.k));
    p.C.resize(size_t(p.ldc) * p.n);
    std::vector<in_t> ha(p.A.size()), hb(p.B.size());
    for (size_t j = 0; j < p.A.size(); ++j) {
      float v = U(gen);
      if constexpr (std::is_same_v<in_t, float>) ha[j] = v;
      else ha[j] = to_bf16(v), v = from_bf16(ha[j]);
      p.A[j] = v;
    }
    for (size_t j = 0; j < p.B.size(); ++j) {
      float v = U(gen);
      if constexpr (std::is_same_v<in_t, float>) hb[j] = v;
      else hb[j] = to_bf16(v), v = from_bf16(hb[j]);
      p.B[j] = v;
    }
    for (auto& x : p.C) x = U(gen);
    cudaMalloc((void**)&dA[i], ha.size() * sizeof(in_t));
    cudaMalloc((void**)&dB[i], hb.size() * sizeof(in_t));
    cudaMalloc((void**)&dC[i], p.C.size() * 4);
    cudaMemcpy(dA[i], ha.data(), ha.size() * sizeof(in_t), cudaMemcpyHostToDevice);
    cudaMemcpy(dB[i], hb.data(), hb.size() * sizeof(in_t), cudaMemcpyHostToDevice);
    cudaMemcpy(dC[i], p.C.data(), p.C.size() * 4, cudaMemcpyHostToDevice);
  }
  std::vector<int64_t> m(count), n(count), k(count), lda(count), ldb(count), ldc(count);
  std::vector<float> alpha(count), beta(count);
  std::vector<char> ta(count), tb(count);
  std::vector<const in_t*> a(count), b(count);
  for (int i = 0; i < count; ++i) {
    m[i] = P[i].m, n[i] = P[i].n, k[i] = P[i].k, lda[i] = P[i].lda, ldb[i] = P[i].ldb, ldc[i] = P[i].ldc;
    alpha[i] = P[i].alpha, beta[i] = P[i].beta, ta[i] = P[i].ta, tb[i] = P[i].tb;
    a[i] = dA[i], b[i] = dB[i];
  }
  blas::SB_Handle::event_t ev;
  if (use_plan) {
    blas::extension::gemm_grouped_plan<in_t> plan(sb, int64_t(count), ta.data(), tb.data(), m.data(), n.data(),
                                                  k.data(), alpha.data(), a.data(), lda.data(), b.data(),
                                                  ldb.data(), beta.data(), dC.data(), ldc.data());
    ev = plan.run(sb);
    sb.wait(ev);
  } else {
    ev = blas::extension::_gemm_grouped(sb, int64_t(count), ta.data(), tb.data(), m.data(), n.data(), k.data(),
                                        alpha.data(), a.data(), lda.data(), b.data(), ldb.data(), beta.data(),
                                        dC.data(), ldc.data());
    sb.wait(ev);
  }
  double worst = 0;
  for (int i = 0; i < count; ++i) {
    const Problem& p = P[i];
    std::vector<float> out(p.C.size());
    cudaMemcpy(out.data(), dC[i], out.size() * 4, cudaMemcpyDeviceToHost);
    for (int64_t c = 0; c < p.n; ++c)
      for (int64_t r = 0; r < p.ldc; ++r) {
        const double got = out[r + c * p.ldc];
        if (r >= p.m) {  // padding rows untouched
          if (got != p.C[r + c * p.ldc]) worst = 1e30;
          continue;
        }
        double acc = 0, mag = 0;
        for (int64_t q2 = 0; q2 < p.k; ++q2) {
          const double av = p.ta == 'n' ? p.A[r + q2 * p.lda] : p.A[q2 + r * p.lda];
          const double bv = p.tb == 'n' ? p.B[q2 + c * p.ldb] : p.B[c + q2 * p.ldb];
          acc += av * bv;
          mag += std::fabs(av * bv);
        }
        const double ref = p.alpha * acc + p.beta * double(p.C[r + c * p.ldc]);
        const double scale = std::fabs(p.alpha) * mag + std::fabs(p.beta * double(p.C[r + c * p.ldc])) + 1e-30;
        worst = std::fmax(worst, std::fabs(got - ref) / scale);
      }
  }
  for (int i = 0; i < count; ++i) cudaFree(dA[i]), cudaFree(dB[i]), cudaFree(dC[i]);
  std::printf("grouped %s %s: max normalised error %.3g\n", std::is_same_v<in_t, float> ? "fp32" : "bf16",
              use_plan ? "plan" : "one-shot", worst);
  return worst < 1e-5 ? 0 : 1;
}

// An event held by the caller keeps its own CUDA event while any number of
// later calls return theirs; released events are reused.
int event_lifetime(cudaStream_t q) {
  blas::SB_Handle sb(q);
  float* d;
  cudaMalloc((void**)&d, 1024 * 4);
  cudaMemset(d, 0, 1024 * 4);
  blas::SB_Handle::event_t held = blas::_scal(sb, 1024, 2.0f, d, 1);
  const cudaEvent_t mine = held[0];
  std::set<cudaEvent_t> later;
  for (int i = 0; i < 200; ++i) {
    blas::SB_Handle::event_t e = blas::_scal(sb, 1024, 1.0f, d, 1);
    later.insert(e[0].get());
  }  // each e is released at the end of its iteration
  sb.wait(held);
  const bool unique = later.count(mine) == 0 && held[0].get() == mine && held[0].is_complete();
  const bool recycled = later.size() <= 2;  // released events come back
  sb.wait();
  cudaFree(d);
  std::printf("event lifetime: held event unique %d, %zu distinct later events\n", int(unique), later.size());
  return (unique && recycled) ? 0 : 1;
}

}  // namespace

int main() {
  cudaStream_t q;
  cudaStreamCreate(&q);
  int bad = 0;
  bad |= run<float>(q, false);
  bad |= run<float>(q, true);
  bad |= run<uint16_t>(q, false);
  bad |= run<uint16_t>(q, true);
  bad |= event_lifetime(q);
  // events outlive their handle: a copy kept past the handle's end stays usable
  blas::SB_Handle::event_t kept;
  {
    blas::SB_Handle sb(q);
    float* d;
    cudaMalloc((void**)&d, 64 * 4);
    kept = blas::_scal(sb, 64, 1.0f, d, 1);
    sb.wait();
    cudaFree(d);
  }
  kept[0].wait();
  cudaStreamDestroy(q);
  std::printf(bad ? "FAILED\n" : "ok\n");
  return bad;
}

// reduce_util.cuh — compensated accumulators shared by the reduction kernels.
#pragma once
#include <cuda_runtime.h>

namespace gb {

__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }

// L2-coherent load of any 4-byte-multiple POD (partials written by other CTAs
// of the same launch).
template <typename T>
__device__ __forceinline__ T ldcg_any(const T* p) {
  static_assert(sizeof(T) % 4 == 0, "ldcg_any needs a 4-byte multiple");
  T r;
  const unsigned int* src = reinterpret_cast<const unsigned int*>(p);
  unsigned int* dst = reinterpret_cast<unsigned int*>(&r);
#pragma unroll
  for (int i = 0; i < int(sizeof(T) / 4); ++i) dst[i] = __ldcg(src + i);
  return r;
}

// Knuth's TwoSum: s + e == a + b exactly, s = RN(a + b).  The _rn intrinsics
// keep the compiler from contracting or reassociating the steps.
template <typename T>
__device__ __forceinline__ T two_sum(T a, T b, T& e) {
  T s = rn_add(a, b);
  T bp = rn_sub(s, a);
  T ap = rn_sub(s, bp);
  e = rn_add(rn_sub(a, ap), rn_sub(b, bp));
  return s;
}

// Compensated running sum (s, c): value = s + c.  FP32 carries the exact
// rounding error of every addition (and, for products, of every multiply,
// Ogita-Rump-Oishi Dot2).  FP64 data uses a plain FP64 sum: its precision
// already exceeds what the FP32 oracle tolerances ask for, and the FP64
// issue rate, not HBM, would bound a compensated FP64 loop on GB300.
template <typename T>
struct CompSum;

template <>
struct CompSum<float> {
  float s, c;
  __device__ static CompSum zero() { return CompSum{0.f, 0.f}; }
  __device__ __forceinline__ void add(float x) {
    float e;
    s = two_sum(s, x, e);
    c = rn_add(c, e);
  }
  __device__ __forceinline__ void add_product(float x, float y) {
    float p = rn_mul(x, y);
    float pe = fmaf(x, y, -p);  // exact error of the product
    float e;
    s = two_sum(s, p, e);
    c = rn_add(c, rn_add(e, pe));
  }
  __device__ __forceinline__ void merge(const CompSum& o) {
    float e;
    s = two_sum(s, o.s, e);
    c = rn_add(c, rn_add(o.c, e));
  }
  __device__ __forceinline__ CompSum shfl_down(int off) const {
    return CompSum{__shfl_down_sync(0xffffffffu, s, off), __shfl_down_sync(0xffffffffu, c, off)};
  }
  __device__ __forceinline__ float value() const { return rn_add(s, c); }
};

template <>
struct CompSum<double> {
  double s, c;
  __device__ static CompSum zero() { return CompSum{0.0, 0.0}; }
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ void add_product(double x, double y) { s = fma(x, y, s); }
  __device__ __forceinline__ void merge(const CompSum& o) {
    double e;
    s = two_sum(s, o.s, e);
    c = c + o.c + e;
  }
  __device__ __forceinline__ CompSum shfl_down(int off) const {
    return CompSum{__shfl_down_sync(0xffffffffu, s, off), __shfl_down_sync(0xffffffffu, c, off)};
  }
  __device__ __forceinline__ double value() const { return s + c; }
};

}  // namespace gb

// blas1.cu — asum, nrm2, dot, iamax, iamin on sm_103a.
//
// One kernel shape serves every reduction: a grid-stride pass with 128-bit
// loads (contiguous, 16-byte aligned data) or strided scalar loads, a
// per-thread accumulator, a fixed-order warp-shuffle + shared-memory block
// combine, one partial per CTA in temp memory, and a last-CTA-done ticket
// whose holder combines the partials in a fixed order and writes the result.
// Nothing waits on another CTA, and the combine order depends only on
// (n, grid), so results are deterministic run to run — unlike the float
// atomics of portBLAS's WGAtomicReduction
// (src/operations/blas1/WGAtomicReduction.hpp:92-138).  A grid of one full
// wave is launched with programmatic dependent launch (common.cuh).
//
// Operator semantics follow src/operations/blas_operators.hpp:149-316 and
// the interface rules of src/interface/blas1_interface.hpp:117-642.
#include <type_traits>
#include <cfloat>
#include <climits>
#include <cmath>

#include "common.cuh"
#include "reduce_util.cuh"

namespace gb {

// --------------------------------------------------------------- operators --
// asum: sum of |x| with a Neumaier-compensated accumulator (float) or a plain
// FP64 one (double: FP64 issue rate is the scarce resource on GB300).
template <typename T>
struct AsumOp {
  using Acc = CompSum<T>;
  __device__ static Acc init() { return Acc::zero(); }
  using Out = T;
  __device__ static void add(Acc& a, T x, T, int64_t) { a.add(fabs(x)); }
  // one 128-bit packet: plain sum of the (at most 4) magnitudes, then one
  // compensated addition
  template <int W>
  __device__ static void add_vec(Acc& a, const T* x, const T*, int64_t) {
    T s = fabs(x[0]);
#pragma unroll
    for (int e = 1; e < W; ++e) s += fabs(x[e]);
    a.add(s);
  }
  __device__ static void combine(Acc& a, const Acc& b) { a.merge(b); }
  __device__ static Acc shfl(const Acc& a, int off) { return a.shfl_down(off); }
  __device__ static void finish(const Acc& a, Out* r) { *r = a.value(); }
};

// dot: Ogita–Rump–Oishi Dot2 — the rounding error of each product is
// recovered exactly with an FMA and carried with the compensated sum.
template <typename T>
struct DotOp {
  using Acc = CompSum<T>;
  __device__ static Acc init() { return Acc::zero(); }
  using Out = T;
  __device__ static void add(Acc& a, T x, T y, int64_t) { a.add_product(x, y); }
  template <int W>
  __device__ static void add_vec(Acc& a, const T* x, const T* y, int64_t) {
#pragma unroll
    for (int e = 0; e < W; ++e) a.add_product(x[e], y[e]);
  }
  __device__ static void combine(Acc& a, const Acc& b) { a.merge(b); }
  __device__ static Acc shfl(const Acc& a, int off) { return a.shfl_down(off); }
  __device__ static void finish(const Acc& a, Out* r) { *r = a.value(); }
};

// nrm2: Blue's three-accumulator scaling (J. Blue, ACM TOMS 4(1) 1978, in the
// form of E. Anderson, "Algorithm 978: Safe Scaling in the Level 1 BLAS",
// ACM TOMS 44(1) 2017): elements below `tsml` are scaled up by `ssml`,
// elements above `tbig` scaled down by `sbig`, so no square over- or
// underflows.  portBLAS squares unscaled (src/interface/blas1_interface.hpp:555-579).
template <typename T>
struct BlueConst;
template <>
struct BlueConst<float> {
  // emin = -125, emax = 128, t = 24 (FLT_MIN_EXP, FLT_MAX_EXP, FLT_MANT_DIG)
  static constexpr float tsml = 0x1p-63f;   // 2^ceil((emin-1)/2)
  static constexpr float tbig = 0x1p+52f;   // 2^floor((emax-t+1)/2)
  static constexpr float ssml = 0x1p+75f;   // 2^-floor((emin-t)/2)
  static constexpr float sbig = 0x1p-76f;   // 2^-ceil((emax+t-1)/2)
};
template <>
struct BlueConst<double> {
  // emin = -1021, emax = 1024, t = 53
  static constexpr double tsml = 0x1p-511;
  static constexpr double tbig = 0x1p+486;
  static constexpr double ssml = 0x1p+537;
  static constexpr double sbig = 0x1p-538;
};

template <typename T>
struct Nrm2Acc {
  CompSum<T> med;
  T sml, big;
  __device__ Nrm2Acc shfl_down(int off) const {
    Nrm2Acc r;
    r.med = med.shfl_down(off);
    r.sml = __shfl_down_sync(0xffffffffu, sml, off);
    r.big = __shfl_down_sync(0xffffffffu, big, off);
    return r;
  }
};

template <typename T>
struct Nrm2Op {
  using Acc = Nrm2Acc<T>;
  using C = BlueConst<T>;
  __device__ static Acc init() {
    Acc a;
    a.med = CompSum<T>::zero();
    a.sml = T(0);
    a.big = T(0);
    return a;
  }
  __device__ static void add(Acc& a, T x, T, int64_t) {
    T ax = fabs(x);
    if (ax > C::tbig) {
      T s = ax * C::sbig;
      a.big = fma(s, s, a.big);
    } else if (ax < C::tsml) {
      T s = ax * C::ssml;
      a.sml = fma(s, s, a.sml);
    } else {
      a.med.add(ax * ax);  // NaN lands here and propagates, as it must
    }
  }
  // one packet: when every |x| is in the medium range (the common case) the
  // squares are summed plainly and added once with compensation
  template <int W>
  __device__ static void add_vec(Acc& a, const T* x, const T* y, int64_t i) {
    T lo = fabs(x[0]), hi = lo;
#pragma unroll
    for (int e = 1; e < W; ++e) {
      lo = fmin(lo, fabs(x[e]));
      hi = fmax(hi, fabs(x[e]));
    }
    if (lo >= C::tsml && hi <= C::tbig) {
      T s = x[0] * x[0];
#pragma unroll
      for (int e = 1; e < W; ++e) s = fma(x[e], x[e], s);
      a.med.add(s);
    } else {
#pragma unroll
      for (int e = 0; e < W; ++e) add(a, x[e], y ? y[e] : T(0), i + e);
    }
  }
  __device__ static void combine(Acc& a, const Acc& b) {
    a.med.merge(b.med);
    a.sml += b.sml;
    a.big += b.big;
  }
  __device__ static Acc shfl(const Acc& a, int off) { return a.shfl_down(off); }
  using Out = T;
  __device__ static void finish(const Acc& a, Out* r);
};

// Final scale-and-sqrt of the three accumulators, in FP64.
__device__ inline double nrm2_finish(const Nrm2Acc<float>& a) {
  using C = BlueConst<float>;
  // FP64 holds the unscaled partial sums of FP32 data without over/underflow.
  double big = double(a.big) / (double(C::sbig) * double(C::sbig));
  double sml = double(a.sml) / (double(C::ssml) * double(C::ssml));
  double med = double(a.med.s) + double(a.med.c);
  return sqrt(big + med + sml);
}

// FP64 data: the three sums are combined the way Anderson's algorithm does,
// keeping the scaled representation until the square root.
__device__ inline double nrm2_finish(const Nrm2Acc<double>& a) {
  using C = BlueConst<double>;
  double amed = a.med.s + a.med.c;
  double abig = a.big, asml = a.sml;
  double scl, sumsq;
  if (abig > 0.0) {
    if (amed > 0.0 || isnan(amed)) abig += (amed * C::sbig) * C::sbig;
    scl = 1.0 / C::sbig;
    sumsq = abig;
  } else if (asml > 0.0) {
    if (amed > 0.0 || isnan(amed)) {
      double ymed = sqrt(amed);
      double ysml = sqrt(asml) / C::ssml;
      double ymin = ysml > ymed ? ymed : ysml;
      double ymax = ysml > ymed ? ysml : ymed;
      scl = 1.0;
      sumsq = ymax * ymax * (1.0 + (ymin / ymax) * (ymin / ymax));
    } else {
      scl = 1.0 / C::ssml;
      sumsq = asml;
    }
  } else {
    scl = 1.0;
    sumsq = amed;
  }
  return scl * sqrt(sumsq);
}

template <typename T>
__device__ void Nrm2Op<T>::finish(const Acc& a, Out* r) {
  *r = T(nrm2_finish(a));
}

// iamax / iamin: (|value|, index) pairs compared exactly as IMaxOperator /
// IMinOperator do (src/operations/blas_operators.hpp:276-316): the larger
// (smaller) |value| wins and equal |values| keep the lower index.  The
// initial pair is (0, INT_MAX) for max and (T max, INT_MAX) for min
// (include/operations/blas_constants.h), so NaN never wins.
constexpr int64_t kNoIndex = INT64_MAX;

template <typename T>
struct IdxAcc {
  T v;
  int64_t i;
  __device__ IdxAcc shfl_down(int off) const {
    IdxAcc r;
    r.v = __shfl_down_sync(0xffffffffu, v, off);
    r.i = __shfl_down_sync(0xffffffffu, (long long)i, off);
    return r;
  }
};

template <typename T, bool IS_MAX>
struct IamaxOp {
  using Acc = IdxAcc<T>;
  // The walk of one thread visits increasing indices, so within a thread a
  // strict comparison keeps the first index of a tie.  The thread-level
  // initial value sits just outside portBLAS's initial tuple: -1 below
  // IMax's 0 (so |x| == 0 still wins) and +inf above IMin's T max (so
  // |x| == T max still wins while inf, like in portBLAS, never does).
  __device__ static Acc init() {
    Acc a;
    a.v = IS_MAX ? T(-1) : T(INFINITY);
    a.i = kNoIndex;
    return a;
  }
  __device__ static bool better(T av, int64_t ai, T bv, int64_t bi) {
    // does (av, ai) beat (bv, bi)?
    if (IS_MAX) return av > bv || (av == bv && ai < bi);
    return av < bv || (av == bv && ai < bi);
  }
  __device__ static void add(Acc& a, T x, T, int64_t idx) {
    T ax = fabs(x);
    if (IS_MAX ? (ax > a.v) : (ax < a.v)) {
      a.v = ax;
      a.i = idx;
    }
  }
  template <int W>
  __device__ static void add_vec(Acc& a, const T* x, const T*, int64_t i) {
#pragma unroll
    for (int e = 0; e < W; ++e) add(a, x[e], T(0), i + e);
  }
  __device__ static void combine(Acc& a, const Acc& b) {
    if (better(b.v, b.i, a.v, a.i)) a = b;
  }
  __device__ static Acc shfl(const Acc& a, int off) { return a.shfl_down(off); }
  using Out = int32_t;
  __device__ static void finish(const Acc& a, Out* r) { *r = a.i == kNoIndex ? INT32_MAX : int32_t(a.i); }
};

// ------------------------------------------------------------------ kernel --
constexpr int kThreads = 512;
constexpr int kUnroll = 4;

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int n = 4;
  __device__ static void unpack(const float4& v, float* o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int n = 2;
  __device__ static void unpack(const double2& v, double* o) { o[0] = v.x; o[1] = v.y; }
};

template <class Op>
__device__ __forceinline__ typename Op::Acc block_reduce(typename Op::Acc a, typename Op::Acc* smem) {
  // fixed-order warp tree, then warp 0 folds the per-warp results in order
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    typename Op::Acc o = Op::shfl(a, off);
    Op::combine(a, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) smem[warp] = a;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  if (warp == 0) {
    a = lane < nw ? smem[lane] : Op::init();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      typename Op::Acc o = Op::shfl(a, off);
      Op::combine(a, o);
    }
  }
  return a;  // valid in thread 0
}

// VEC: x (and y) contiguous and 16-byte aligned; otherwise strided scalar
// loads from the view base (negative increments allowed).
// Resident CTAs per SM the kernel is compiled for (and the grid is sized
// to): 4 x 512 threads (32 registers) for FP32, 2 for FP64; nrm2's three
// accumulators, iamax's value-index pairs and dot's two streams need more
// than 32 registers (at 32, iamax and dot spilled), so 3.
template <class Op, typename T>
struct Blas1Occupancy {
  static constexpr int kCtas = sizeof(T) == 4 ? 4 : 2;
};
template <>
struct Blas1Occupancy<Nrm2Op<float>, float> {
  static constexpr int kCtas = 3;
};
template <bool IS_MAX>
struct Blas1Occupancy<IamaxOp<float, IS_MAX>, float> {
  static constexpr int kCtas = 3;
};
template <>
struct Blas1Occupancy<DotOp<float>, float> {
  static constexpr int kCtas = 3;
};

// L2 prefetch of a CTA's first batch: kUnroll runs of blockDim.x 16-byte
// vectors of x (and y) from vector blockIdx.x * blockDim.x on, nthreads apart.
__device__ __noinline__ void prefetch_first_batch(const void* x, const void* y, int64_t nv, int64_t nthreads) {
  for (int u = 0; u < kUnroll; ++u) {
    const int64_t v = int64_t(blockIdx.x) * blockDim.x + u * nthreads;
    if (v >= nv) break;
    const int64_t left = nv - v;
    const uint32_t bytes = uint32_t(left < int64_t(blockDim.x) ? left : int64_t(blockDim.x)) * 16u;
    prefetch_l2_bulk(static_cast<const uint8_t*>(x) + v * 16, bytes);
    if (y) prefetch_l2_bulk(static_cast<const uint8_t*>(y) + v * 16, bytes);
  }
}

template <class Op, typename T, bool VEC, bool HAS_Y>
__global__ void __launch_bounds__(kThreads, Blas1Occupancy<Op, T>::kCtas) blas1_reduce(int64_t n, const T* __restrict__ x, int64_t incx,
                                                         const T* __restrict__ y, int64_t incy,
                                                         typename Op::Acc* __restrict__ partials,
                                                         unsigned int* __restrict__ ticket,
                                                         typename Op::Out* __restrict__ result) {
  using Acc = typename Op::Acc;
  __shared__ Acc smem[kThreads / 32];
  __shared__ bool is_last;
  pdl_trigger();
  const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t nthreads = int64_t(gridDim.x) * blockDim.x;
  // warm L2 with the CTA's first batch while the previous kernel drains (a
  // call, so its registers stay out of the main loop's 32)
  if (VEC && threadIdx.x == 0) prefetch_first_batch(x, HAS_Y ? y : nullptr, n / Vec16<T>::n, nthreads);
  pdl_wait();  // before any global memory load
  Acc acc = Op::init();
  if (VEC) {
    using V = Vec16<T>;
    using VT = typename V::type;
    constexpr int W = V::n;
    const int64_t nv = n / W;
    const VT* xv = reinterpret_cast<const VT*>(x);
    const VT* yv = reinterpret_cast<const VT*>(y);
    int64_t v = tid;
    // kUnroll independent 128-bit loads in flight per thread
    for (; v + (kUnroll - 1) * nthreads < nv; v += kUnroll * nthreads) {
      VT xr[kUnroll], yr[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        xr[u] = __ldcs(xv + v + u * nthreads);
        if (HAS_Y) yr[u] = __ldcs(yv + v + u * nthreads);
      }
#pragma unroll
      for (int u = 0; u < kUnroll; ++u) {
        T xe[W], ye[W];
        V::unpack(xr[u], xe);
        if (HAS_Y) V::unpack(yr[u], ye);
        Op::template add_vec<W>(acc, xe, HAS_Y ? ye : nullptr, (v + u * nthreads) * W);
      }
    }
    for (; v < nv; v += nthreads) {
      T xe[W], ye[W];
      V::unpack(__ldcs(xv + v), xe);
      if (HAS_Y) V::unpack(__ldcs(yv + v), ye);
      Op::template add_vec<W>(acc, xe, HAS_Y ? ye : nullptr, v * W);
    }
    // scalar tail, taken by the threads that follow in grid order
    for (int64_t i = nv * W + tid; i < n; i += nthreads) Op::add(acc, x[i], HAS_Y ? y[i] : T(0), i);
  } else {
    // strided: asum and nrm2 keep kUnroll independent loads in flight per
    // thread (nrm2 with incx 2 on 2^25: 70.7 -> 51.5 us); dot and iamax /
    // iamin keep one (unrolled, iamax spilled at its register cap and dot
    // measured no gain).  Each thread visits its indices in increasing order.
    constexpr int SU = (HAS_Y || std::is_same<typename Op::Acc, IdxAcc<T>>::value) ? 1 : kUnroll;
    const T* xb = vec_base(x, n, incx);
    const T* yb = HAS_Y ? vec_base(y, n, incy) : nullptr;
    int64_t i = tid;
    for (; i + (SU - 1) * nthreads < n; i += SU * nthreads) {
      T xr[SU], yr[SU];
#pragma unroll
      for (int u = 0; u < SU; ++u) {
        xr[u] = xb[(i + u * nthreads) * incx];
        yr[u] = HAS_Y ? yb[(i + u * nthreads) * incy] : T(0);
      }
#pragma unroll
      for (int u = 0; u < SU; ++u) Op::add(acc, xr[u], yr[u], i + u * nthreads);
    }
    for (; i < n; i += nthreads) Op::add(acc, xb[i * incx], HAS_Y ? yb[i * incy] : T(0), i);
  }
  acc = block_reduce<Op>(acc, smem);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = acc;
    __threadfence();
    unsigned int prev = atomicAdd(ticket, 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return;
  // Last CTA: fold the per-CTA partials in index order (strided by thread,
  // then the fixed block tree).
  __threadfence();
  Acc a = Op::init();
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) Op::combine(a, ldcg_any(partials + b));
  __syncthreads();
  a = block_reduce<Op>(a, smem);
  if (threadIdx.x == 0) {
    Op::finish(a, result);
    *ticket = 0u;  // leave the ticket zeroed for the next call
  }
}

__global__ void fill_index(int32_t* result, int32_t v) { *result = v; }

// ------------------------------------------------------------------- host --
template <class Op, typename T, bool HAS_Y>
gbblas_status_t launch_reduce(gbblas_handle_t h, int64_t n, const T* x, int64_t incx, const T* y, int64_t incy,
                              typename Op::Out* result) {
  using Acc = typename Op::Acc;
  const bool vec = incx == 1 && aligned16(x) && (!HAS_Y || (incy == 1 && aligned16(y)));
  const int64_t per_block = int64_t(kThreads) * (vec ? 16 / int(sizeof(T)) : 1) * kUnroll;
  int64_t blocks = cdiv(n > 0 ? n : 1, per_block);
  const int64_t cap = int64_t(h->sm_count) * Blas1Occupancy<Op, T>::kCtas;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  void* tmp = nullptr;
  GB_TRY(temp_acquire(h, sizeof(Acc) * blocks, &tmp));
  Acc* partials = static_cast<Acc*>(tmp);
  // a full wave (every SM at its CTA limit) may be placed early
  const bool early = blocks == cap;
  const cudaError_t e =
      vec ? launch_pdl(early, blas1_reduce<Op, T, true, HAS_Y>, dim3(unsigned(blocks)), dim3(kThreads), 0, h->stream,
                       n, x, incx, y, incy, partials, h->tickets, result)
          : launch_pdl(early, blas1_reduce<Op, T, false, HAS_Y>, dim3(unsigned(blocks)), dim3(kThreads), 0,
                       h->stream, n, x, incx, y, incy, partials, h->tickets, result);
  if (e != cudaSuccess) return cuda_fail(e, "blas1_reduce");
  return after_launch("blas1_reduce");
}

template <typename T>
gbblas_status_t asum_impl(gbblas_handle_t h, int64_t n, const T* x, int64_t incx, T* result) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "asum: null handle");
  if (!result || (n > 0 && !x)) return fail(GBBLAS_STATUS_INVALID_ARG, "asum: null pointer");
  if (n < 0) n = 0;
  return launch_reduce<AsumOp<T>, T, false>(h, n, x, incx, nullptr, 0, result);
}

template <typename T>
gbblas_status_t nrm2_impl(gbblas_handle_t h, int64_t n, const T* x, int64_t incx, T* result) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "nrm2: null handle");
  if (!result || (n > 0 && !x)) return fail(GBBLAS_STATUS_INVALID_ARG, "nrm2: null pointer");
  if (n < 0) n = 0;
  return launch_reduce<Nrm2Op<T>, T, false>(h, n, x, incx, nullptr, 0, result);
}

template <typename T>
gbblas_status_t dot_impl(gbblas_handle_t h, int64_t n, const T* x, int64_t incx, const T* y, int64_t incy,
                         T* result) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "dot: null handle");
  if (n <= 0) return GBBLAS_STATUS_SUCCESS;  // result untouched (blas1_interface.hpp:623)
  if (!result || !x || !y) return fail(GBBLAS_STATUS_INVALID_ARG, "dot: null pointer");
  return launch_reduce<DotOp<T>, T, true>(h, n, x, incx, y, incy, result);
}

template <typename T, bool IS_MAX>
gbblas_status_t iamax_impl(gbblas_handle_t h, int64_t n, const T* x, int64_t incx, int32_t* result) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "iamax/iamin: null handle");
  if (!result) return fail(GBBLAS_STATUS_INVALID_ARG, "iamax/iamin: null result");
  if (incx < 0 || n < 0) {  // blas1_interface.hpp:375-378
    fill_index<<<1, 1, 0, h->stream>>>(result, 0);
    return after_launch("fill_index");
  }
  if (n > 0 && !x) return fail(GBBLAS_STATUS_INVALID_ARG, "iamax/iamin: null x");
  return launch_reduce<IamaxOp<T, IS_MAX>, T, false>(h, n, x, incx, nullptr, 0, result);
}

template <typename R, typename F>
gbblas_status_t sync_call(gbblas_handle_t h, R* host_result, F&& enqueue) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "sync: null handle");
  if (!host_result) return fail(GBBLAS_STATUS_INVALID_ARG, "sync: null host result");
  void* dres = nullptr;
  GB_CUDA_TRY(cudaMallocAsync(&dres, 16, h->stream));
  GB_CUDA_TRY(cudaMemsetAsync(dres, 0, 16, h->stream));
  gbblas_status_t s = enqueue(static_cast<R*>(dres));
  if (s == GBBLAS_STATUS_SUCCESS) {
    cudaError_t e = cudaMemcpyAsync(h->pinned, dres, sizeof(R), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) s = cuda_fail(e, "sync result copy");
    else *host_result = *static_cast<R*>(h->pinned);
  }
  cudaFreeAsync(dres, h->stream);
  return s;
}

}  // namespace gb

using namespace gb;

extern "C" {

gbblas_status_t gbblas_sasum(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, float* r) {
  clear_error();
  return asum_impl(h, n, x, incx, r);
}
gbblas_status_t gbblas_dasum(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, double* r) {
  clear_error();
  return asum_impl(h, n, x, incx, r);
}
gbblas_status_t gbblas_snrm2(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, float* r) {
  clear_error();
  return nrm2_impl(h, n, x, incx, r);
}
gbblas_status_t gbblas_dnrm2(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, double* r) {
  clear_error();
  return nrm2_impl(h, n, x, incx, r);
}
gbblas_status_t gbblas_sdot(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, const float* y,
                            int64_t incy, float* r) {
  clear_error();
  return dot_impl(h, n, x, incx, y, incy, r);
}
gbblas_status_t gbblas_ddot(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, const double* y,
                            int64_t incy, double* r) {
  clear_error();
  return dot_impl(h, n, x, incx, y, incy, r);
}
gbblas_status_t gbblas_isamax(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, int32_t* r) {
  clear_error();
  return iamax_impl<float, true>(h, n, x, incx, r);
}
gbblas_status_t gbblas_isamin(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, int32_t* r) {
  clear_error();
  return iamax_impl<float, false>(h, n, x, incx, r);
}
gbblas_status_t gbblas_idamax(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, int32_t* r) {
  clear_error();
  return iamax_impl<double, true>(h, n, x, incx, r);
}
gbblas_status_t gbblas_idamin(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, int32_t* r) {
  clear_error();
  return iamax_impl<double, false>(h, n, x, incx, r);
}

gbblas_status_t gbblas_sasum_sync(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, float* hr) {
  clear_error();
  return sync_call<float>(h, hr, [&](float* d) { return asum_impl(h, n, x, incx, d); });
}
gbblas_status_t gbblas_dasum_sync(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, double* hr) {
  clear_error();
  return sync_call<double>(h, hr, [&](double* d) { return asum_impl(h, n, x, incx, d); });
}
gbblas_status_t gbblas_snrm2_sync(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, float* hr) {
  clear_error();
  return sync_call<float>(h, hr, [&](float* d) { return nrm2_impl(h, n, x, incx, d); });
}
gbblas_status_t gbblas_dnrm2_sync(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, double* hr) {
  clear_error();
  return sync_call<double>(h, hr, [&](double* d) { return nrm2_impl(h, n, x, incx, d); });
}
gbblas_status_t gbblas_sdot_sync(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, const float* y,
                                 int64_t incy, float* hr) {
  clear_error();
  return sync_call<float>(h, hr, [&](float* d) { return dot_impl(h, n, x, incx, y, incy, d); });
}
gbblas_status_t gbblas_ddot_sync(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, const double* y,
                                 int64_t incy, double* hr) {
  clear_error();
  return sync_call<double>(h, hr, [&](double* d) { return dot_impl(h, n, x, incx, y, incy, d); });
}
gbblas_status_t gbblas_isamax_sync(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, int32_t* hr) {
  clear_error();
  return sync_call<int32_t>(h, hr, [&](int32_t* d) { return iamax_impl<float, true>(h, n, x, incx, d); });
}
gbblas_status_t gbblas_isamin_sync(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, int32_t* hr) {
  clear_error();
  return sync_call<int32_t>(h, hr, [&](int32_t* d) { return iamax_impl<float, false>(h, n, x, incx, d); });
}
gbblas_status_t gbblas_idamax_sync(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, int32_t* hr) {
  clear_error();
  return sync_call<int32_t>(h, hr, [&](int32_t* d) { return iamax_impl<double, true>(h, n, x, incx, d); });
}
gbblas_status_t gbblas_idamin_sync(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, int32_t* hr) {
  clear_error();
  return sync_call<int32_t>(h, hr, [&](int32_t* d) { return iamax_impl<double, false>(h, n, x, incx, d); });
}

}  // extern "C"

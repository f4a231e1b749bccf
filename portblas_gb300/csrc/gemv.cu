// gemv.cu — y <- alpha*op(A)*x + beta*y on sm_103a.
//
// Replaces portBLAS's two-kernel GEMV (partial dot products into temp
// memory, then SumMatrixColumns + ScalarOp/Assign:
// src/interface/blas2_interface.hpp:68-217, src/operations/blas2/gemv.hpp:40-371)
// with one HBM-bound sweep whose split partials are folded by the last CTA of
// each output tile; the alpha/beta epilogue is fused.  beta == 0 never reads
// y (blas2_interface.hpp:205-211); trans 'n'/'N' is the normal sweep and any
// other character the transposed one (blas2_interface.hpp:1163-1192).
#include "stream_sweep.cuh"

namespace gb {

template <typename T>
struct GemvPolicy {
  using Acc = T;
  T alpha, beta;
  T* yb;  // base of the y view
  int64_t incy;
  __device__ __forceinline__ Acc init() const { return T(0); }
  __device__ __forceinline__ void add(Acc& a, T v, T x) const { a = fma(v, x, a); }
  __device__ __forceinline__ void merge(Acc& a, const Acc& b) const { a += b; }
  __device__ __forceinline__ Acc shfl_down(const Acc& a, int off) const { return __shfl_down_sync(0xffffffffu, a, off); }
  __device__ __forceinline__ void finish(const Acc& a, int64_t i) const {
    T* yp = yb + i * incy;
    T r = alpha * a;
    if (beta != T(0)) r = fma(beta, *yp, r);
    *yp = r;
  }
};

// ------------------------------------------------- transposed, warp per column --
// y[j] = alpha * sum_i A[i + j*lda] x[i] + beta * y[j] with one warp per
// column: lane l reads the 16-byte vectors l, l + 32, ... of the column (and
// of x, which every warp reads, from L1), kGtwUnroll in flight, then a fixed
// shuffle tree; no partial sums, no fold, the same order on every run.  The
// grid is at most one wave (kGtwCtas CTAs of 8 warps per SM, 64 registers,
// no spills) and column j goes to warp (j / grid) of CTA (j % grid), so the
// CTAs get the same number of columns to within one.  Taken for x
// contiguous and, with 16-byte-aligned columns, between a quarter and two
// columns per warp of the wave; with columns the TMA cannot address
// (ALIGNED false below) from a quarter column per warp up; otherwise the TMA
// column sweep
// (fewer columns leave too few loads in flight, more leave a ragged last
// round: 16384^2 measured 160 us here against 154 for the sweep).  Not
// launched early: placed early, its CTAs shared SMs with the GEMV before it
// and the nine-op step ran 51 us longer, though each op alone was faster.
// ALIGNED: columns and x 16-byte aligned (x read as 16-byte vectors too);
// otherwise each column's first elements up to its first 16-byte boundary
// are read one per lane, the rest of the column as 16-byte vectors, and x
// one element per lane (x is in L1 after the first columns): a leading
// dimension that is not a multiple of 16 bytes keeps the vector loads of A.
constexpr int kGtwUnroll = 4, kGtwCtas = 4;

template <typename T, bool ALIGNED>
__global__ void __launch_bounds__(kMvThreads, kGtwCtas)
    gemv_t_warp_cols(GemvPolicy<T> pol, int64_t m, int64_t n, const T* __restrict__ A, int64_t lda,
                     const T* __restrict__ x) {
  using V = typename Pack16<T>::V;
  constexpr int W = Pack16<T>::n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t step = int64_t(kMvWarps) * gridDim.x;
  const int64_t first = int64_t(warp) * gridDim.x + blockIdx.x;
  for (int64_t j = first; j < n; j += step) {
    const T* col = A + j * lda;
    T acc = T(0);
    int64_t head = 0;  // elements before the column's first 16-byte boundary
    if (!ALIGNED) {
      head = int64_t(((16 - (reinterpret_cast<uintptr_t>(col) & 15)) & 15) / sizeof(T));
      if (head > m) head = m;
      if (lane < head) acc = col[lane] * x[lane];
    }
    const V* av = reinterpret_cast<const V*>(col + head);
    const T* xh = x + head;
    const int64_t nv = (m - head) / W;  // whole vectors after the head
    int64_t v = lane;
    for (; v + 32 * (kGtwUnroll - 1) < nv; v += 32 * kGtwUnroll) {
      V a[kGtwUnroll];
#pragma unroll
      for (int u = 0; u < kGtwUnroll; ++u) a[u] = __ldcs(av + v + 32 * u);
      if (ALIGNED) {
        V b[kGtwUnroll];
#pragma unroll
        for (int u = 0; u < kGtwUnroll; ++u) b[u] = __ldg(reinterpret_cast<const V*>(xh) + v + 32 * u);
#pragma unroll
        for (int u = 0; u < kGtwUnroll; ++u) {
          T ae[W], be[W];
          Pack16<T>::get(a[u], ae);
          Pack16<T>::get(b[u], be);
#pragma unroll
          for (int e = 0; e < W; ++e) acc = fma(ae[e], be[e], acc);
        }
      } else {
#pragma unroll
        for (int u = 0; u < kGtwUnroll; ++u) {
          T ae[W];
          Pack16<T>::get(a[u], ae);
#pragma unroll
          for (int e = 0; e < W; ++e) acc = fma(ae[e], __ldg(xh + (v + 32 * u) * W + e), acc);
        }
      }
    }
    for (; v < nv; v += 32) {
      T ae[W];
      Pack16<T>::get(__ldcs(av + v), ae);
#pragma unroll
      for (int e = 0; e < W; ++e) acc = fma(ae[e], __ldg(xh + v * W + e), acc);
    }
    for (int64_t i = head + nv * W + lane; i < m; i += 32) acc = fma(col[i], x[i], acc);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if (lane == 0) pol.finish(acc, j);
  }
}

template <typename T>
gbblas_status_t gemv_impl(gbblas_handle_t h, char trans, int64_t m, int64_t n, T alpha, const T* a, int64_t lda,
                          const T* x, int64_t incx, T beta, T* y, int64_t incy) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "gemv: null handle");
  if (m < 0 || n < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "gemv: negative dimension");
  if (incx == 0 || incy == 0) return fail(GBBLAS_STATUS_INVALID_ARG, "gemv: zero increment");
  if (lda < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "gemv: negative lda");
  const bool tr = !(trans == 'n' || trans == 'N');
  const int64_t xlen = tr ? m : n, ylen = tr ? n : m;
  if (ylen == 0) return GBBLAS_STATUS_SUCCESS;
  if (!y || (xlen > 0 && (!a || !x))) return fail(GBBLAS_STATUS_INVALID_ARG, "gemv: null pointer");
  GemvPolicy<T> pol{alpha, beta, vec_base(y, ylen, incy), incy};
  const T* xb = vec_base(x, xlen, incx);
  constexpr int RPT = 16 / sizeof(T);
  const bool vec = (lda % RPT == 0) && aligned16(a);
  if (!tr) {
    gbblas_status_t st = GBBLAS_STATUS_SUCCESS;
    if (try_rows_sweep_tma<GemvPolicy<T>, T, true>(h, pol, m, n, a, lda, xb, incx, &st)) return st;
    SweepPlan p = plan_rows(m, n, h->sm_count, sizeof(T));
    T* partials = nullptr;
    if (p.split > 1) {
      void* tmp;
      GB_TRY(temp_acquire(h, sizeof(T) * p.split * m, &tmp));
      partials = static_cast<T*>(tmp);
    }
    dim3 grid(unsigned(p.tiles), unsigned(p.split));
    if (vec)
      rows_sweep<GemvPolicy<T>, T, true, true><<<grid, kMvThreads, 0, h->stream>>>(
          pol, m, n, a, lda, xb, incx, p.per_split, partials, h->tickets);
    else
      rows_sweep<GemvPolicy<T>, T, false, true><<<grid, kMvThreads, 0, h->stream>>>(
          pol, m, n, a, lda, xb, incx, p.per_split, partials, h->tickets);
    return after_launch("gemv_n");
  }
  {
    // one column per warp where that fits in one wave, else the full wave
    const int64_t slots = int64_t(kGtwCtas) * h->sm_count, warps = slots * kMvWarps;
    const int64_t want = cdiv(n, int64_t(kMvWarps));
    const int64_t grid = want < slots ? want : slots;
    // aligned A: the warp kernel up to two columns per warp (the TMA sweep
    // beyond); A the TMA cannot address (unaligned lda): the warp kernel at
    // any width, against the element-wise sweep otherwise
    if (incx == 1 && m > 0 && 4 * n >= warps) {
      if (vec && aligned16(x) && n <= 2 * warps) {
        gemv_t_warp_cols<T, true><<<unsigned(grid), kMvThreads, 0, h->stream>>>(pol, m, n, a, lda, x);
        return after_launch("gemv_t_warp_cols");
      }
      if (!vec) {
        gemv_t_warp_cols<T, false><<<unsigned(grid), kMvThreads, 0, h->stream>>>(pol, m, n, a, lda, x);
        return after_launch("gemv_t_warp_cols");
      }
    }
    gbblas_status_t st = GBBLAS_STATUS_SUCCESS;
    if (try_cols_sweep_tma<GemvPolicy<T>, T, true>(h, pol, m, n, a, lda, xb, incx, &st)) return st;
  }
  SweepPlan p = plan_cols(m, n, h->sm_count, sizeof(T));
  const int64_t chunk_cols = int64_t(kMaxTickets) * p.cols_per_cta;
  T* partials = nullptr;
  if (p.split > 1) {
    void* tmp;
    GB_TRY(temp_acquire(h, sizeof(T) * p.split * (n < chunk_cols ? n : chunk_cols), &tmp));
    partials = static_cast<T*>(tmp);
  }
  const size_t smem = ((p.per_split * sizeof(T) + 15) & ~size_t(15)) + sizeof(T) * p.cols_per_cta;
  for (int64_t c0 = 0; c0 < n; c0 += chunk_cols) {
    const int64_t nc = n - c0 < chunk_cols ? n - c0 : chunk_cols;
    GemvPolicy<T> pc = pol;
    pc.yb = pol.yb + c0 * incy;
    dim3 grid(unsigned(cdiv(nc, p.cols_per_cta)), unsigned(p.split));
    if (vec)
      cols_sweep<GemvPolicy<T>, T, true, true><<<grid, kMvThreads, smem, h->stream>>>(
          pc, m, nc, a + c0 * lda, lda, xb, incx, p.per_split, p.cols_per_cta, partials, h->tickets);
    else
      cols_sweep<GemvPolicy<T>, T, false, true><<<grid, kMvThreads, smem, h->stream>>>(
          pc, m, nc, a + c0 * lda, lda, xb, incx, p.per_split, p.cols_per_cta, partials, h->tickets);
    GB_TRY(after_launch("gemv_t"));
  }
  return GBBLAS_STATUS_SUCCESS;
}

}  // namespace gb

using namespace gb;

extern "C" {

gbblas_status_t gbblas_sgemv(gbblas_handle_t h, char trans, int64_t m, int64_t n, float alpha, const float* a,
                             int64_t lda, const float* x, int64_t incx, float beta, float* y, int64_t incy) {
  clear_error();
  return gemv_impl<float>(h, trans, m, n, alpha, a, lda, x, incx, beta, y, incy);
}

gbblas_status_t gbblas_dgemv(gbblas_handle_t h, char trans, int64_t m, int64_t n, double alpha, const double* a,
                             int64_t lda, const double* x, int64_t incx, double beta, double* y, int64_t incy) {
  clear_error();
  return gemv_impl<double>(h, trans, m, n, alpha, a, lda, x, incx, beta, y, incy);
}

}  // extern "C"

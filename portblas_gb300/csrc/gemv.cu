// gemv.cu — y <- alpha*op(A)*x + beta*y on sm_103a.
//
// Replaces portBLAS's two-kernel GEMV (partial dot products into temp
// memory, then SumMatrixColumns + ScalarOp/Assign:
// src/interface/blas2_interface.hpp:68-217, src/operations/blas2/gemv.hpp:40-371)
// with one HBM-bound sweep whose split partials are folded by the last CTA of
// each output tile; the alpha/beta epilogue is fused.  beta == 0 never reads
// y (blas2_interface.hpp:205-211); trans 'n'/'N' is the normal sweep and any
// other character the transposed one (blas2_interface.hpp:1163-1192).
// Short, wide A (at most 32 lanes x 16 bytes of rows) and, for 'n', tall A
// of at most 32 columns take kernels shaped for them (matvec.cuh:
// rows_narrow, cols_thread, cols_lanes, rows_tall), so that every warp load
// stays a contiguous run of the matrix.
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

// GEMV 'n' with at most narrow_rows<T>() rows: rows_narrow over about four CTAs
// per SM, each over at least four whole load rounds of columns.
template <typename T>
static gbblas_status_t gemv_n_narrow(gbblas_handle_t h, const GemvPolicy<T>& pol, int64_t m, int64_t n,
                                     const T* a, int64_t lda, const T* xb, int64_t incx, bool vec) {
  constexpr int RPT = 16 / sizeof(T);
  int lpc_log2 = 0;
  while ((int64_t(1) << lpc_log2) * RPT < m) ++lpc_log2;
  const int64_t round = int64_t(32 >> lpc_log2) * kMvWarps;  // columns of one load round of a CTA
  const int64_t cols = n > 0 ? n : 1;
  int64_t per = cdiv(cdiv(cols, 4 * int64_t(h->sm_count)), round) * round;
  if (per < 4 * round) per = 4 * round;
  const int64_t grid = cdiv(cols, per);
  if (grid > INT32_MAX) return fail(GBBLAS_STATUS_UNSUPPORTED, "gemv: too many columns");
  T* partials = nullptr;
  if (grid > 1) {
    void* tmp;
    GB_TRY(temp_acquire(h, sizeof(T) * grid * m, &tmp));
    partials = static_cast<T*>(tmp);
  }
  if (vec)
    rows_narrow<GemvPolicy<T>, T, true, true><<<unsigned(grid), kMvThreads, 0, h->stream>>>(
        pol, int(m), n, a, lda, xb, incx, lpc_log2, per, partials, h->tickets);
  else
    rows_narrow<GemvPolicy<T>, T, false, true><<<unsigned(grid), kMvThreads, 0, h->stream>>>(
        pol, int(m), n, a, lda, xb, incx, lpc_log2, per, partials, h->tickets);
  return after_launch("gemv_n_narrow");
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
    if (m <= narrow_rows<T>()) return gemv_n_narrow<T>(h, pol, m, n, a, lda, xb, incx, vec);
    if (n <= kTallCols && m >= 64 * int64_t(h->sm_count)) {
      // tall, narrow A: a warp per 32 x RPT rows over every column (rows_tall)
      const int64_t grid = cdiv(m, int64_t(kMvThreads) * (16 / sizeof(T)));
      if (grid > INT32_MAX) return fail(GBBLAS_STATUS_UNSUPPORTED, "gemv: too many rows");
      if (vec)
        rows_tall<GemvPolicy<T>, T, true, true><<<unsigned(grid), kMvThreads, 0, h->stream>>>(pol, m, int(n), a, lda,
                                                                                               xb, incx);
      else
        rows_tall<GemvPolicy<T>, T, false, true><<<unsigned(grid), kMvThreads, 0, h->stream>>>(pol, m, int(n), a,
                                                                                                lda, xb, incx);
      return after_launch("gemv_n_tall");
    }
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
  if (m <= kThreadRows) {
    // at most kThreadRows rows: one thread per column (cols_thread; 8 x 2^22
    // 25.6 us against 39.5 for cols_lanes)
    const int64_t grid = cdiv(n, kMvThreads);
    if (grid > INT32_MAX) return fail(GBBLAS_STATUS_UNSUPPORTED, "gemv: too many columns");
    if (vec)
      cols_thread<GemvPolicy<T>, T, true, true><<<unsigned(grid), kMvThreads, 0, h->stream>>>(pol, int(m), n, a,
                                                                                               lda, xb, incx);
    else
      cols_thread<GemvPolicy<T>, T, false, true><<<unsigned(grid), kMvThreads, 0, h->stream>>>(pol, int(m), n, a,
                                                                                                lda, xb, incx);
    return after_launch("gemv_t_narrow");
  }
  if (m <= narrow_rows<T>()) {
    // up to 32 lanes x 16 bytes of rows: a few lanes per column (cols_lanes;
    // 64 x 2^20 186 -> 65 us against a warp per column), up to 8 CTAs per SM
    int lpc_log2 = 0;
    while ((int64_t(1) << lpc_log2) * RPT < m) ++lpc_log2;
    const int64_t per_cta = int64_t(32 >> lpc_log2) * kMvWarps;
    int64_t grid = cdiv(n, per_cta);
    if (grid > 8 * int64_t(h->sm_count)) grid = 8 * int64_t(h->sm_count);
    if (vec)
      cols_lanes<GemvPolicy<T>, T, true, true><<<unsigned(grid), kMvThreads, 0, h->stream>>>(pol, int(m), n, a, lda,
                                                                                              xb, incx, lpc_log2);
    else
      cols_lanes<GemvPolicy<T>, T, false, true><<<unsigned(grid), kMvThreads, 0, h->stream>>>(pol, int(m), n, a,
                                                                                               lda, xb, incx, lpc_log2);
    return after_launch("gemv_t_narrow");
  }
  {
    // aligned columns up to two per warp of the wave: a CTA per column
    // group, its warps over equal row ranges (cols_cta in matvec.cuh; 8192^2
    // 45.0 -> 42.2 us against one warp per column, whose warps got one or
    // two columns; the TMA sweep's rounds end evenly only at full widths such
    // as 16384^2); columns the TMA cannot address at any width: one warp per
    // column (cols_warp; 8191^2: 49 us against 100 for the element-wise
    // sweep).  Neither is launched early: placed early, the CTAs shared SMs
    // with the GEMV before it and the nine-op step ran 51 us longer.
    if (incx == 1) {
      gbblas_status_t st = GBBLAS_STATUS_SUCCESS;
      if (try_cols_warp<GemvPolicy<T>, T, true>(h, pol, m, n, a, lda, x, true, &st)) return st;
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

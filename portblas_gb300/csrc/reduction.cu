// reduction.cu — blas::extension::_reduction<op, T> on sm_103a.
//
// inner: out(j) = fold_i in(i, j)  (one value per column, 1 x cols)
// outer: out(i) = fold_j in(i, j)  (one value per row, rows x 1)
// (include/operations/extension/reduction.h:40, doc/Reduction.md).
//
// Operators and their initial values follow src/operations/blas_operators.hpp:149-274
// and include/operations/blas_constants.h:111-127: Add 0, Product 1, Max
// lowest(), Min max(), AbsoluteAdd sum of |x|, Mean = Add then divide by the
// reduced length (src/interface/extension_interface.hpp:46-53).  Add, Mean
// and AbsoluteAdd carry a compensated sum.  portBLAS runs one or two
// Reduction launches with a temp buffer (extension_interface.hpp:344-409);
// here each direction is one sweep (matvec.cuh) whose split partials are
// folded by the last CTA of each output tile.
//
// Element (i, j) is in[i + j*ld].  portBLAS computes the column offset as
// (ld / rows) * rows * j (src/operations/extension/reduction.hpp:44, 128-134),
// which equals ld * j whenever ld is a multiple of rows — the only layout
// its tests use.
#include <cfloat>

#include "stream_sweep.cuh"

namespace gb {

template <typename T>
struct RedAcc {
  T s, c;
};

template <typename T>
struct Lim;
template <>
struct Lim<float> {
  __device__ static float max() { return FLT_MAX; }
};
template <>
struct Lim<double> {
  __device__ static double max() { return DBL_MAX; }
};

template <typename T, int OP>
struct RedPolicy {
  using Acc = RedAcc<T>;
  T* out;
  int64_t nred;  // reduced length (Mean divisor)
  __device__ __forceinline__ Acc init() const {
    switch (OP) {
      case GBBLAS_OP_PRODUCT: return Acc{T(1), T(0)};
      case GBBLAS_OP_MAX: return Acc{-Lim<T>::max(), T(0)};
      case GBBLAS_OP_MIN: return Acc{Lim<T>::max(), T(0)};
      default: return Acc{T(0), T(0)};
    }
  }
  __device__ __forceinline__ void add(Acc& a, T v, T) const {
    switch (OP) {
      case GBBLAS_OP_PRODUCT: a.s = a.s * v; break;
      case GBBLAS_OP_MAX: a.s = (a.s > v) ? a.s : v; break;
      case GBBLAS_OP_MIN: a.s = (a.s < v) ? a.s : v; break;
      default: {
        T x = OP == GBBLAS_OP_ABS_ADD ? fabs(v) : v;
        T e;
        a.s = two_sum(a.s, x, e);
        a.c += e;
      }
    }
  }
  __device__ __forceinline__ void merge(Acc& a, const Acc& b) const {
    switch (OP) {
      case GBBLAS_OP_PRODUCT: a.s = a.s * b.s; break;
      case GBBLAS_OP_MAX: a.s = (a.s > b.s) ? a.s : b.s; break;
      case GBBLAS_OP_MIN: a.s = (a.s < b.s) ? a.s : b.s; break;
      default: {
        T e;
        a.s = two_sum(a.s, b.s, e);
        a.c = a.c + b.c + e;
      }
    }
  }
  __device__ __forceinline__ Acc shfl_down(const Acc& a, int off) const {
    return Acc{__shfl_down_sync(0xffffffffu, a.s, off), __shfl_down_sync(0xffffffffu, a.c, off)};
  }
  __device__ __forceinline__ void finish(const Acc& a, int64_t i) const {
    switch (OP) {
      case GBBLAS_OP_PRODUCT:
      case GBBLAS_OP_MAX:
      case GBBLAS_OP_MIN: out[i] = a.s; break;
      case GBBLAS_OP_MEAN: out[i] = (a.s + a.c) / T(nred); break;
      default: out[i] = a.s + a.c;
    }
  }
};

template <typename T, int OP>
gbblas_status_t reduction_op(gbblas_handle_t h, int dim, const T* in, int64_t ld, T* out, int64_t rows,
                             int64_t cols) {
  constexpr int RPT = 16 / sizeof(T);
  const bool vec = (ld % RPT == 0) && aligned16(in);
  using P = RedPolicy<T, OP>;
  using Acc = typename P::Acc;
  if (dim == GBBLAS_DIM_OUTER) {
    P pol{out, cols};
    gbblas_status_t st = GBBLAS_STATUS_SUCCESS;
    if (try_rows_sweep_tma<P, T, false>(h, pol, rows, cols, in, ld, static_cast<const T*>(nullptr), 0, &st))
      return st;
    SweepPlan p = plan_rows(rows, cols, h->sm_count, sizeof(T));
    Acc* partials = nullptr;
    if (p.split > 1) {
      void* tmp;
      GB_TRY(temp_acquire(h, sizeof(Acc) * p.split * rows, &tmp));
      partials = static_cast<Acc*>(tmp);
    }
    dim3 grid(unsigned(p.tiles), unsigned(p.split));
    if (vec)
      rows_sweep<P, T, true, false><<<grid, kMvThreads, 0, h->stream>>>(pol, rows, cols, in, ld, nullptr, 0,
                                                                        p.per_split, partials, h->tickets);
    else
      rows_sweep<P, T, false, false><<<grid, kMvThreads, 0, h->stream>>>(pol, rows, cols, in, ld, nullptr, 0,
                                                                         p.per_split, partials, h->tickets);
    return after_launch("reduction_outer");
  }
  {
    P pol{out, rows};
    gbblas_status_t st = GBBLAS_STATUS_SUCCESS;
    if (try_cols_sweep_tma<P, T, false>(h, pol, rows, cols, in, ld, static_cast<const T*>(nullptr), 0, &st))
      return st;
    // columns TMA cannot address: one warp per column with 16-byte loads
    // after each column's head (cols_warp in matvec.cuh)
    if (try_cols_warp<P, T, false>(h, pol, rows, cols, in, ld, static_cast<const T*>(nullptr), false, &st))
      return st;
  }
  SweepPlan p = plan_cols(rows, cols, h->sm_count, sizeof(T));
  const int64_t chunk_cols = int64_t(kMaxTickets) * p.cols_per_cta;
  Acc* partials = nullptr;
  if (p.split > 1) {
    void* tmp;
    GB_TRY(temp_acquire(h, sizeof(Acc) * p.split * (cols < chunk_cols ? cols : chunk_cols), &tmp));
    partials = static_cast<Acc*>(tmp);
  }
  const size_t smem = ((p.per_split * sizeof(T) + 15) & ~size_t(15)) + sizeof(Acc) * p.cols_per_cta;
  for (int64_t c0 = 0; c0 < cols; c0 += chunk_cols) {
    const int64_t nc = cols - c0 < chunk_cols ? cols - c0 : chunk_cols;
    P pol{out + c0, rows};
    dim3 grid(unsigned(cdiv(nc, p.cols_per_cta)), unsigned(p.split));
    if (vec)
      cols_sweep<P, T, true, false><<<grid, kMvThreads, smem, h->stream>>>(
          pol, rows, nc, in + c0 * ld, ld, nullptr, 0, p.per_split, p.cols_per_cta, partials, h->tickets);
    else
      cols_sweep<P, T, false, false><<<grid, kMvThreads, smem, h->stream>>>(
          pol, rows, nc, in + c0 * ld, ld, nullptr, 0, p.per_split, p.cols_per_cta, partials, h->tickets);
    GB_TRY(after_launch("reduction_inner"));
  }
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status_t reduction_impl(gbblas_handle_t h, int op, int dim, const T* in, int64_t ld, T* out, int64_t rows,
                               int64_t cols) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "reduction: null handle");
  if (rows < 0 || cols < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "reduction: negative dimension");
  if (dim != GBBLAS_DIM_INNER && dim != GBBLAS_DIM_OUTER)
    return fail(GBBLAS_STATUS_INVALID_ARG, "reduction: unknown reduction_dim");
  if (ld < rows) return fail(GBBLAS_STATUS_INVALID_ARG, "reduction: ld < rows");
  if (rows == 0 || cols == 0) return GBBLAS_STATUS_SUCCESS;
  if (!in || !out) return fail(GBBLAS_STATUS_INVALID_ARG, "reduction: null pointer");
  switch (op) {
    case GBBLAS_OP_ADD: return reduction_op<T, GBBLAS_OP_ADD>(h, dim, in, ld, out, rows, cols);
    case GBBLAS_OP_PRODUCT: return reduction_op<T, GBBLAS_OP_PRODUCT>(h, dim, in, ld, out, rows, cols);
    case GBBLAS_OP_MAX: return reduction_op<T, GBBLAS_OP_MAX>(h, dim, in, ld, out, rows, cols);
    case GBBLAS_OP_MIN: return reduction_op<T, GBBLAS_OP_MIN>(h, dim, in, ld, out, rows, cols);
    case GBBLAS_OP_ABS_ADD: return reduction_op<T, GBBLAS_OP_ABS_ADD>(h, dim, in, ld, out, rows, cols);
    case GBBLAS_OP_MEAN: return reduction_op<T, GBBLAS_OP_MEAN>(h, dim, in, ld, out, rows, cols);
  }
  return fail(GBBLAS_STATUS_UNSUPPORTED, "reduction: unknown operator");
}

}  // namespace gb

using namespace gb;

extern "C" {

gbblas_status_t gbblas_sreduction(gbblas_handle_t h, int op, int dim, const float* in, int64_t ld, float* out,
                                  int64_t rows, int64_t cols) {
  clear_error();
  return reduction_impl<float>(h, op, dim, in, ld, out, rows, cols);
}

gbblas_status_t gbblas_dreduction(gbblas_handle_t h, int op, int dim, const double* in, int64_t ld, double* out,
                                  int64_t rows, int64_t cols) {
  clear_error();
  return reduction_impl<double>(h, op, dim, in, ld, out, rows, cols);
}

}  // extern "C"

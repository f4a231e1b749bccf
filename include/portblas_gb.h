/*
 * portblas_gb.h — header-only C++ shim that re-creates portBLAS's `blas::`
 * interface for the hot path on top of the gbblas C ABI (gbblas.h).
 *
 * Source written against portBLAS compiles unchanged for these calls: the
 * function names, template shapes, argument order and meaning follow
 *   include/interface/blas1_interface.h   (_asum, _nrm2, _dot, _iamax, _iamin,
 *                                          _scal, _axpy, _copy, _sdsdot)
 *   include/interface/blas2_interface.h   (_gemv)
 *   include/interface/blas3_interface.h   (_gemm, _gemm_batched, _gemm_strided_batched, _symm;
 *                                          extension::_gemm_grouped has no portBLAS counterpart)
 *   include/interface/extension_interface.h (extension::_reduction, _omatcopy, _transpose)
 * and the errors are the same exception types (std::invalid_argument,
 * blas::unsupported_exception).  Differences a caller can observe:
 *   - SB_Handle wraps a cudaStream_t instead of a sycl::queue, and buffers are
 *     device pointers (portBLAS's USM mode); there is no BufferIterator.
 *   - event_t is a vector of blas::event, each owning one recorded CUDA event
 *     (converts to cudaEvent_t).  Each call makes its stream wait on the
 *     dependency events and returns one event recorded after its work.  An
 *     event stays valid, and refers to its own point in the stream, for as
 *     long as a copy of it is held; its cudaEvent_t is reused for a later
 *     call only after the last copy is gone (also after the handle is gone).
 *   - the async BLAS-1 reductions overwrite the result (portBLAS adds into it).
 */
#ifndef PORTBLAS_GB_H
#define PORTBLAS_GB_H

#include <cuda_runtime_api.h>

#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "gbblas.h"

namespace blas {

enum class transpose_type : char { Normal = 'n', Transposed = 't', Conjugate = 'c' };
enum class gemm_batch_type_t : int { strided = 0, interleaved = 1 };
enum class reduction_dim_t : int { inner = 0, outer = 1 };

/* include/blas_meta.h:225-235 */
class unsupported_exception : public std::runtime_error {
 public:
  explicit unsupported_exception(const std::string& what) : std::runtime_error(what) {}
};

/* operator tags of extension::_reduction (src/operations/blas_operators.hpp:149-274) */
struct AddOperator { static constexpr int code = GBBLAS_OP_ADD; };
struct ProductOperator { static constexpr int code = GBBLAS_OP_PRODUCT; };
struct MaxOperator { static constexpr int code = GBBLAS_OP_MAX; };
struct MinOperator { static constexpr int code = GBBLAS_OP_MIN; };
struct AbsoluteAddOperator { static constexpr int code = GBBLAS_OP_ABS_ADD; };
struct MeanOperator { static constexpr int code = GBBLAS_OP_MEAN; };

namespace detail {
inline void check(gbblas_status_t s) {
  if (s == GBBLAS_STATUS_SUCCESS) return;
  std::string msg = gbblas_last_error();
  if (msg.empty()) msg = gbblas_status_string(s);
  switch (s) {
    case GBBLAS_STATUS_INVALID_ARG: throw std::invalid_argument(msg);
    case GBBLAS_STATUS_UNSUPPORTED: throw unsupported_exception(msg);
    default: throw std::runtime_error(msg);
  }
}
template <typename C>
using elem_t = std::remove_cv_t<std::remove_pointer_t<C>>;
}  // namespace detail

namespace detail {
/* Recycled CUDA events of one handle.  Shared by the handle and by every
 * event it handed out, so it lives until the last of them is gone. */
class EventPool {
 public:
  ~EventPool() {
    for (cudaEvent_t e : free_) cudaEventDestroy(e);
  }
  cudaEvent_t acquire() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (!free_.empty()) {
        cudaEvent_t e = free_.back();
        free_.pop_back();
        return e;
      }
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
      throw std::runtime_error("SB_Handle: cudaEventCreate failed");
    return e;
  }
  void release(cudaEvent_t e) {
    std::lock_guard<std::mutex> lk(mu_);
    free_.push_back(e);
  }

 private:
  std::mutex mu_;
  std::vector<cudaEvent_t> free_;
};
}  // namespace detail

/* One point in a handle's stream, as a sycl::event is one submitted command
 * group.  Copies share the CUDA event; it goes back to its handle's pool when
 * the last copy is destroyed. */
class event {
 public:
  event() = default;
  explicit event(std::shared_ptr<CUevent_st> e) : e_(std::move(e)) {}
  cudaEvent_t get() const { return e_.get(); }
  operator cudaEvent_t() const { return e_.get(); }
  void wait() const {
    if (e_ && cudaEventSynchronize(e_.get()) != cudaSuccess) throw std::runtime_error("blas::event::wait failed");
  }
  /* sycl::event::get_info<command_execution_status> counterpart: true once
   * the work before the event has finished. */
  bool is_complete() const { return !e_ || cudaEventQuery(e_.get()) == cudaSuccess; }

 private:
  std::shared_ptr<CUevent_st> e_;
};

/* blas::SB_Handle (include/sb_handle/portblas_handle.h:46-200) over a CUDA stream. */
class SB_Handle {
 public:
  using event_t = std::vector<event>;

  explicit SB_Handle(cudaStream_t stream = nullptr) : stream_(stream), pool_(std::make_shared<detail::EventPool>()) {
    detail::check(gbblas_handle_create(static_cast<void*>(stream), &h_));
  }
  ~SB_Handle() { gbblas_handle_destroy(h_); }
  SB_Handle(const SB_Handle&) = delete;
  SB_Handle& operator=(const SB_Handle&) = delete;

  cudaStream_t get_queue() const { return stream_; }
  gbblas_handle_t native() const { return h_; }
  void wait() { detail::check(gbblas_wait(h_)); }
  void wait(const event_t& evs) {
    for (const event& e : evs) e.wait();
  }
  void set_sgemm_mode(gbblas_sgemm_mode_t m) { detail::check(gbblas_set_sgemm_mode(h_, m)); }

  // stream waits for the dependencies; returns an event after `status`'s work
  void depend(const event_t& deps) {
    for (const event& e : deps)
      if (e.get() && cudaStreamWaitEvent(stream_, e.get(), 0) != cudaSuccess)
        throw std::runtime_error("SB_Handle: cudaStreamWaitEvent failed");
  }
  event_t done(gbblas_status_t status) {
    detail::check(status);
    cudaEvent_t raw = pool_->acquire();
    if (cudaEventRecord(raw, stream_) != cudaSuccess) {
      pool_->release(raw);
      throw std::runtime_error("SB_Handle: cudaEventRecord failed");
    }
    std::shared_ptr<detail::EventPool> pool = pool_;
    return event_t{event(std::shared_ptr<CUevent_st>(raw, [pool](CUevent_st* p) { pool->release(p); }))};
  }

 private:
  cudaStream_t stream_;
  gbblas_handle_t h_ = nullptr;
  std::shared_ptr<detail::EventPool> pool_;
};

/* ------------------------------------------------------------------ BLAS-3 */
template <typename sb_handle_t, typename container_0_t, typename container_1_t, typename container_2_t,
          typename element_t, typename index_t>
typename sb_handle_t::event_t _gemm(sb_handle_t& sb, char ta, char tb, index_t M, index_t N, index_t K,
                                    element_t alpha, container_0_t a, index_t lda, container_1_t b, index_t ldb,
                                    element_t beta, container_2_t c, index_t ldc,
                                    const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<container_2_t>;
  sb.depend(deps);
  if constexpr (std::is_same_v<T, float>)
    return sb.done(gbblas_sgemm(sb.native(), ta, tb, M, N, K, float(alpha), a, lda, b, ldb, float(beta), c, ldc));
  else if constexpr (std::is_same_v<T, double>)
    return sb.done(gbblas_dgemm(sb.native(), ta, tb, M, N, K, double(alpha), a, lda, b, ldb, double(beta), c, ldc));
  else
    throw unsupported_exception("_gemm: element type not supported");
}

template <typename sb_handle_t, typename container_0_t, typename container_1_t, typename container_2_t,
          typename element_t, typename index_t>
typename sb_handle_t::event_t _gemm_batched(sb_handle_t& sb, char ta, char tb, index_t M, index_t N, index_t K,
                                            element_t alpha, container_0_t a, index_t lda, container_1_t b,
                                            index_t ldb, element_t beta, container_2_t c, index_t ldc,
                                            index_t batch_size,
                                            gemm_batch_type_t batch_type = gemm_batch_type_t::strided,
                                            const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<container_2_t>;
  sb.depend(deps);
  if constexpr (std::is_same_v<T, float>)
    return sb.done(gbblas_sgemm_batched(sb.native(), ta, tb, M, N, K, float(alpha), a, lda, b, ldb, float(beta), c,
                                        ldc, batch_size, int(batch_type)));
  else if constexpr (std::is_same_v<T, double>)
    return sb.done(gbblas_dgemm_batched(sb.native(), ta, tb, M, N, K, double(alpha), a, lda, b, ldb, double(beta),
                                        c, ldc, batch_size, int(batch_type)));
  else
    throw unsupported_exception("_gemm_batched: element type not supported");
}

template <typename sb_handle_t, typename container_0_t, typename container_1_t, typename container_2_t,
          typename element_t, typename index_t>
typename sb_handle_t::event_t _gemm_strided_batched(sb_handle_t& sb, char ta, char tb, index_t M, index_t N,
                                                    index_t K, element_t alpha, container_0_t a, index_t lda,
                                                    index_t stridea, container_1_t b, index_t ldb, index_t strideb,
                                                    element_t beta, container_2_t c, index_t ldc, index_t stridec,
                                                    index_t batch_size,
                                                    const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<container_2_t>;
  sb.depend(deps);
  if constexpr (std::is_same_v<T, float>)
    return sb.done(gbblas_sgemm_strided_batched(sb.native(), ta, tb, M, N, K, float(alpha), a, lda, stridea, b, ldb,
                                                strideb, float(beta), c, ldc, stridec, batch_size));
  else if constexpr (std::is_same_v<T, double>)
    return sb.done(gbblas_dgemm_strided_batched(sb.native(), ta, tb, M, N, K, double(alpha), a, lda, stridea, b,
                                                ldb, strideb, double(beta), c, ldc, stridec, batch_size));
  else
    throw unsupported_exception("_gemm_strided_batched: element type not supported");
}

/* _symm: include/interface/blas3_interface.h:135-145 */
template <typename sb_handle_t, typename container_0_t, typename container_1_t, typename container_2_t,
          typename element_t, typename index_t>
typename sb_handle_t::event_t _symm(sb_handle_t& sb, char side, char uplo, index_t M, index_t N, element_t alpha,
                                    container_0_t a, index_t lda, container_1_t b, index_t ldb, element_t beta,
                                    container_2_t c, index_t ldc, const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<container_2_t>;
  sb.depend(deps);
  if constexpr (std::is_same_v<T, float>)
    return sb.done(gbblas_ssymm(sb.native(), side, uplo, M, N, float(alpha), a, lda, b, ldb, float(beta), c, ldc));
  else if constexpr (std::is_same_v<T, double>)
    return sb.done(gbblas_dsymm(sb.native(), side, uplo, M, N, double(alpha), a, lda, b, ldb, double(beta), c, ldc));
  else
    throw unsupported_exception("_symm: element type not supported");
}

/* ------------------------------------------------------------------ BLAS-2 */
template <typename sb_handle_t, typename index_t, typename element_t, typename container_t0,
          typename container_t1, typename increment_t, typename container_t2>
typename sb_handle_t::event_t _gemv(sb_handle_t& sb, char trans, index_t M, index_t N, element_t alpha,
                                    container_t0 a, index_t lda, container_t1 x, increment_t incx, element_t beta,
                                    container_t2 y, increment_t incy,
                                    const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<container_t2>;
  sb.depend(deps);
  if constexpr (std::is_same_v<T, float>)
    return sb.done(gbblas_sgemv(sb.native(), trans, M, N, float(alpha), a, lda, x, incx, float(beta), y, incy));
  else if constexpr (std::is_same_v<T, double>)
    return sb.done(gbblas_dgemv(sb.native(), trans, M, N, double(alpha), a, lda, x, incx, double(beta), y, incy));
  else
    throw unsupported_exception("_gemv: element type not supported");
}

/* ------------------------------------------------------------------ BLAS-1 */
#define PORTBLAS_GB_RED1(NAME)                                                                               \
  template <typename sb_handle_t, typename container_0_t, typename container_1_t, typename index_t,           \
            typename increment_t>                                                                            \
  typename sb_handle_t::event_t _##NAME(sb_handle_t& sb, index_t N, container_0_t x, increment_t incx,        \
                                        container_1_t rs, const typename sb_handle_t::event_t& deps = {}) {   \
    using T = detail::elem_t<container_0_t>;                                                                 \
    sb.depend(deps);                                                                                          \
    if constexpr (std::is_same_v<T, float>)                                                                  \
      return sb.done(gbblas_s##NAME(sb.native(), N, x, incx, rs));                                           \
    else if constexpr (std::is_same_v<T, double>)                                                            \
      return sb.done(gbblas_d##NAME(sb.native(), N, x, incx, rs));                                           \
    else                                                                                                      \
      throw unsupported_exception(#NAME ": element type not supported");                                     \
  }                                                                                                           \
  template <typename sb_handle_t, typename container_t, typename index_t, typename increment_t>              \
  detail::elem_t<container_t> _##NAME(sb_handle_t& sb, index_t N, container_t x, increment_t incx,           \
                                      const typename sb_handle_t::event_t& deps = {}) {                      \
    using T = detail::elem_t<container_t>;                                                                   \
    sb.depend(deps);                                                                                          \
    T r{};                                                                                                    \
    if constexpr (std::is_same_v<T, float>)                                                                  \
      detail::check(gbblas_s##NAME##_sync(sb.native(), N, x, incx, &r));                                     \
    else if constexpr (std::is_same_v<T, double>)                                                            \
      detail::check(gbblas_d##NAME##_sync(sb.native(), N, x, incx, &r));                                     \
    else                                                                                                      \
      throw unsupported_exception(#NAME ": element type not supported");                                     \
    return r;                                                                                                 \
  }

/* _asum: include/interface/blas1_interface.h:631-637 (async), :979-984 (sync) */
PORTBLAS_GB_RED1(asum)
/* _nrm2: include/interface/blas1_interface.h:712-718 (async), :995-1000 (sync) */
PORTBLAS_GB_RED1(nrm2)
#undef PORTBLAS_GB_RED1

/* _dot: include/interface/blas1_interface.h:582-588 (async), :903-909 (sync) */
template <typename sb_handle_t, typename container_0_t, typename container_1_t, typename container_2_t,
          typename index_t, typename increment_t>
typename sb_handle_t::event_t _dot(sb_handle_t& sb, index_t N, container_0_t x, increment_t incx,
                                   container_1_t y, increment_t incy, container_2_t rs,
                                   const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<container_0_t>;
  sb.depend(deps);
  if constexpr (std::is_same_v<T, float>)
    return sb.done(gbblas_sdot(sb.native(), N, x, incx, y, incy, rs));
  else if constexpr (std::is_same_v<T, double>)
    return sb.done(gbblas_ddot(sb.native(), N, x, incx, y, incy, rs));
  else
    throw unsupported_exception("_dot: element type not supported");
}
template <typename sb_handle_t, typename container_0_t, typename container_1_t, typename index_t,
          typename increment_t>
detail::elem_t<container_0_t> _dot(sb_handle_t& sb, index_t N, container_0_t x, increment_t incx, container_1_t y,
                                   increment_t incy, const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<container_0_t>;
  sb.depend(deps);
  T r{};
  if constexpr (std::is_same_v<T, float>)
    detail::check(gbblas_sdot_sync(sb.native(), N, x, incx, y, incy, &r));
  else if constexpr (std::is_same_v<T, double>)
    detail::check(gbblas_ddot_sync(sb.native(), N, x, incx, y, incy, &r));
  else
    throw unsupported_exception("_dot: element type not supported");
  return r;
}

/* _iamax / _iamin: include/interface/blas1_interface.h:646-666 (async, int
 * result), :949-968 (sync) */
#define PORTBLAS_GB_IAM(NAME, S, D)                                                                          \
  template <typename sb_handle_t, typename container_t, typename ContainerI, typename index_t,                 \
            typename increment_t>                                                                            \
  typename sb_handle_t::event_t NAME(sb_handle_t& sb, index_t N, container_t x, increment_t incx,            \
                                     ContainerI rs, const typename sb_handle_t::event_t& deps = {}) {        \
    using T = detail::elem_t<container_t>;                                                                   \
    static_assert(sizeof(detail::elem_t<ContainerI>) == 4, #NAME ": the index result is 32-bit");            \
    sb.depend(deps);                                                                                          \
    int32_t* r = reinterpret_cast<int32_t*>(rs);                                                             \
    if constexpr (std::is_same_v<T, float>)                                                                  \
      return sb.done(S(sb.native(), N, x, incx, r));                                                         \
    else if constexpr (std::is_same_v<T, double>)                                                            \
      return sb.done(D(sb.native(), N, x, incx, r));                                                         \
    else                                                                                                      \
      throw unsupported_exception(#NAME ": element type not supported");                                     \
  }                                                                                                           \
  template <typename sb_handle_t, typename container_t, typename index_t, typename increment_t>              \
  index_t NAME(sb_handle_t& sb, index_t N, container_t x, increment_t incx,                                  \
               const typename sb_handle_t::event_t& deps = {}) {                                             \
    using T = detail::elem_t<container_t>;                                                                   \
    sb.depend(deps);                                                                                          \
    int32_t r = 0;                                                                                            \
    if constexpr (std::is_same_v<T, float>)                                                                  \
      detail::check(S##_sync(sb.native(), N, x, incx, &r));                                                  \
    else if constexpr (std::is_same_v<T, double>)                                                            \
      detail::check(D##_sync(sb.native(), N, x, incx, &r));                                                  \
    else                                                                                                      \
      throw unsupported_exception(#NAME ": element type not supported");                                     \
    return static_cast<index_t>(r);                                                                          \
  }
PORTBLAS_GB_IAM(_iamax, gbblas_isamax, gbblas_idamax)
PORTBLAS_GB_IAM(_iamin, gbblas_isamin, gbblas_idamin)
#undef PORTBLAS_GB_IAM

/* _scal: include/interface/blas1_interface.h:697-701 */
template <typename sb_handle_t, typename element_t, typename container_0_t, typename index_t,
          typename increment_t>
typename sb_handle_t::event_t _scal(sb_handle_t& sb, index_t N, element_t alpha, container_0_t x, increment_t incx,
                                    const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<container_0_t>;
  sb.depend(deps);
  if constexpr (std::is_same_v<T, float>)
    return sb.done(gbblas_sscal(sb.native(), N, float(alpha), x, incx));
  else if constexpr (std::is_same_v<T, double>)
    return sb.done(gbblas_dscal(sb.native(), N, double(alpha), x, incx));
  else
    throw unsupported_exception("_scal: element type not supported");
}

/* _axpy: include/interface/blas1_interface.h:536-541 */
template <typename sb_handle_t, typename element_t, typename container_0_t, typename container_1_t,
          typename index_t, typename increment_t>
typename sb_handle_t::event_t _axpy(sb_handle_t& sb, index_t N, element_t alpha, container_0_t x, increment_t incx,
                                    container_1_t y, increment_t incy,
                                    const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<container_1_t>;
  sb.depend(deps);
  if constexpr (std::is_same_v<T, float>)
    return sb.done(gbblas_saxpy(sb.native(), N, float(alpha), x, incx, y, incy));
  else if constexpr (std::is_same_v<T, double>)
    return sb.done(gbblas_daxpy(sb.native(), N, double(alpha), x, incx, y, incy));
  else
    throw unsupported_exception("_axpy: element type not supported");
}

/* _copy: include/interface/blas1_interface.h:556-560 */
template <typename sb_handle_t, typename index_t, typename container_0_t, typename increment_t,
          typename container_1_t>
typename sb_handle_t::event_t _copy(sb_handle_t& sb, index_t N, container_0_t x, increment_t incx, container_1_t y,
                                    increment_t incy, const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<container_1_t>;
  sb.depend(deps);
  if constexpr (std::is_same_v<T, float>)
    return sb.done(gbblas_scopy(sb.native(), N, x, incx, y, incy));
  else if constexpr (std::is_same_v<T, double>)
    return sb.done(gbblas_dcopy(sb.native(), N, x, incx, y, incy));
  else
    throw unsupported_exception("_copy: element type not supported");
}

/* _sdsdot: include/interface/blas1_interface.h:615-620 (async), :935-940 (sync) */
template <typename sb_handle_t, typename container_0_t, typename container_1_t, typename container_2_t,
          typename index_t, typename increment_t>
typename sb_handle_t::event_t _sdsdot(sb_handle_t& sb, index_t N, float sbv, container_0_t x, increment_t incx,
                                      container_1_t y, increment_t incy, container_2_t rs,
                                      const typename sb_handle_t::event_t& deps = {}) {
  sb.depend(deps);
  return sb.done(gbblas_sdsdot(sb.native(), N, sbv, x, incx, y, incy, rs));
}
template <typename sb_handle_t, typename container_0_t, typename container_1_t, typename index_t,
          typename increment_t>
float _sdsdot(sb_handle_t& sb, index_t N, float sbv, container_0_t x, increment_t incx, container_1_t y,
              increment_t incy, const typename sb_handle_t::event_t& deps = {}) {
  sb.depend(deps);
  float* d = nullptr;
  if (cudaMallocAsync(reinterpret_cast<void**>(&d), sizeof(float), sb.get_queue()) != cudaSuccess)
    throw std::runtime_error("_sdsdot: device allocation failed");
  gbblas_status_t st = gbblas_sdsdot(sb.native(), N, sbv, x, incx, y, incy, d);
  float r = 0.f;
  if (st == GBBLAS_STATUS_SUCCESS)
    cudaMemcpyAsync(&r, d, sizeof(float), cudaMemcpyDeviceToHost, sb.get_queue());
  cudaFreeAsync(d, sb.get_queue());
  cudaStreamSynchronize(sb.get_queue());
  detail::check(st);
  return r;
}

/* --------------------------------------------------------------- extension */
namespace extension {
/* _omatcopy: include/interface/extension_interface.h:188-198 */
template <typename sb_handle_t, typename element_t, typename index_t, typename in_t, typename out_t>
typename sb_handle_t::event_t _omatcopy(sb_handle_t& sb, char trans, index_t m, index_t n, element_t alpha,
                                        in_t in_memory, index_t ld_in, out_t out_memory, index_t ld_out,
                                        const typename sb_handle_t::event_t& deps = {}) {
  using T = detail::elem_t<out_t>;
  sb.depend(deps);
  if constexpr (std::is_same_v<T, float>)
    return sb.done(gbblas_somatcopy(sb.native(), trans, m, n, float(alpha), in_memory, ld_in, out_memory, ld_out));
  else if constexpr (std::is_same_v<T, double>)
    return sb.done(gbblas_domatcopy(sb.native(), trans, m, n, double(alpha), in_memory, ld_in, out_memory, ld_out));
  else
    throw unsupported_exception("_omatcopy: element type not supported");
}

/* _transpose in place: include/interface/extension_interface.h:416-423 */
template <typename element_t, typename sb_handle_t, typename index_t, typename in_t>
typename sb_handle_t::event_t _transpose(sb_handle_t& sb, index_t m, index_t n, in_t A, index_t ld_in, index_t ld_out,
                                         const typename sb_handle_t::event_t& deps = {}) {
  sb.depend(deps);
  if constexpr (std::is_same_v<element_t, float>)
    return sb.done(gbblas_stranspose_inplace(sb.native(), m, n, A, ld_in, ld_out));
  else if constexpr (std::is_same_v<element_t, double>)
    return sb.done(gbblas_dtranspose_inplace(sb.native(), m, n, A, ld_in, ld_out));
  else
    throw unsupported_exception("_transpose: element type not supported");
}

/* _transpose out of place: include/interface/extension_interface.h:443-450 */
template <typename element_t, typename sb_handle_t, typename index_t, typename in_t, typename out_t>
typename sb_handle_t::event_t _transpose(sb_handle_t& sb, index_t m, index_t n, in_t A, index_t ld_a, out_t B,
                                         index_t ld_b, const typename sb_handle_t::event_t& deps = {}) {
  sb.depend(deps);
  if constexpr (std::is_same_v<element_t, float>)
    return sb.done(gbblas_stranspose(sb.native(), m, n, A, ld_a, B, ld_b));
  else if constexpr (std::is_same_v<element_t, double>)
    return sb.done(gbblas_dtranspose(sb.native(), m, n, A, ld_a, B, ld_b));
  else
    throw unsupported_exception("_transpose: element type not supported");
}
/* Uneven batched GEMM.  No portBLAS counterpart: portBLAS batches only
 * problems of one size (_gemm_batched, include/interface/blas3_interface.h:
 * 97-109).  `group_count` independent problems of any sizes,
 * C_i <- alpha_i op_i(A_i) op_i(B_i) + beta_i C_i, run as one persistent
 * tensor-core launch with FP32 accumulation.  A and B are float, or any
 * 2-byte type holding bfloat16 bits (__nv_bfloat16, uint16_t); C is float.
 * transa/transb hold one 'n'/'t'/'c' per problem; every other argument is an
 * array of group_count host values. */
namespace grouped {
template <typename in_t>
constexpr int grouped_dtype() {
  static_assert(std::is_same_v<in_t, float> || sizeof(in_t) == 2,
                "_gemm_grouped: A and B must be float or 2-byte bfloat16");
  return std::is_same_v<in_t, float> ? GBBLAS_DTYPE_F32 : GBBLAS_DTYPE_BF16;
}
/* host copies of the per-problem arrays in the C ABI's types */
struct GroupedArgs {
  std::vector<int64_t> m, n, k, lda, ldb, ldc;
  std::vector<float> alpha, beta;
  std::vector<const void*> a, b;
  template <typename index_t, typename element_t, typename in_t>
  GroupedArgs(index_t count, const index_t* m_, const index_t* n_, const index_t* k_, const element_t* alpha_,
              const in_t* const* a_, const index_t* lda_, const in_t* const* b_, const index_t* ldb_,
              const element_t* beta_, const index_t* ldc_) {
    if (count < 0) throw std::invalid_argument("_gemm_grouped: negative group count");
    const size_t c = size_t(count);
    if (c && (!m_ || !n_ || !k_ || !alpha_ || !a_ || !lda_ || !b_ || !ldb_ || !beta_ || !ldc_))
      throw std::invalid_argument("_gemm_grouped: null argument array");
    m.assign(m_, m_ + c), n.assign(n_, n_ + c), k.assign(k_, k_ + c);
    lda.assign(lda_, lda_ + c), ldb.assign(ldb_, ldb_ + c), ldc.assign(ldc_, ldc_ + c);
    alpha.assign(alpha_, alpha_ + c), beta.assign(beta_, beta_ + c);
    a.assign(a_, a_ + c), b.assign(b_, b_ + c);
  }
};
}  // namespace grouped

template <typename sb_handle_t, typename in_t, typename index_t, typename element_t>
typename sb_handle_t::event_t _gemm_grouped(sb_handle_t& sb, index_t group_count, const char* transa,
                                            const char* transb, const index_t* m, const index_t* n, const index_t* k,
                                            const element_t* alpha, const in_t* const* a, const index_t* lda,
                                            const in_t* const* b, const index_t* ldb, const element_t* beta,
                                            float* const* c, const index_t* ldc,
                                            const typename sb_handle_t::event_t& deps = {}) {
  grouped::GroupedArgs g(group_count, m, n, k, alpha, a, lda, b, ldb, beta, ldc);
  sb.depend(deps);
  return sb.done(gbblas_gemm_grouped(sb.native(), grouped::grouped_dtype<in_t>(), int64_t(group_count), transa,
                                     transb, g.m.data(), g.n.data(), g.k.data(), g.alpha.data(), g.a.data(),
                                     g.lda.data(), g.b.data(), g.ldb.data(), g.beta.data(), c, g.ldc.data()));
}

/* A reusable _gemm_grouped: the problem table goes to the device once, and
 * each run() replays one CUDA graph.  Pointers and sizes are fixed at
 * construction; the data behind them may change between runs. */
template <typename in_t>
class gemm_grouped_plan {
 public:
  template <typename sb_handle_t, typename index_t, typename element_t>
  gemm_grouped_plan(sb_handle_t& sb, index_t group_count, const char* transa, const char* transb, const index_t* m,
                    const index_t* n, const index_t* k, const element_t* alpha, const in_t* const* a,
                    const index_t* lda, const in_t* const* b, const index_t* ldb, const element_t* beta,
                    float* const* c, const index_t* ldc) {
    grouped::GroupedArgs g(group_count, m, n, k, alpha, a, lda, b, ldb, beta, ldc);
    ::blas::detail::check(gbblas_grouped_plan_create(sb.native(), grouped::grouped_dtype<in_t>(), int64_t(group_count), transa,
                                             transb, g.m.data(), g.n.data(), g.k.data(), g.alpha.data(),
                                             g.a.data(), g.lda.data(), g.b.data(), g.ldb.data(), g.beta.data(), c,
                                             g.ldc.data(), &plan_));
  }
  ~gemm_grouped_plan() { gbblas_grouped_plan_destroy(plan_); }
  gemm_grouped_plan(const gemm_grouped_plan&) = delete;
  gemm_grouped_plan& operator=(const gemm_grouped_plan&) = delete;

  template <typename sb_handle_t>
  typename sb_handle_t::event_t run(sb_handle_t& sb, const typename sb_handle_t::event_t& deps = {}) {
    sb.depend(deps);
    return sb.done(gbblas_grouped_plan_run(sb.native(), plan_));
  }

 private:
  gbblas_grouped_plan_t plan_ = nullptr;
};

/* include/interface/extension_interface.h:453-462 */
template <typename operator_t, typename element_t, typename sb_handle_t, typename input_t, typename output_t,
          typename index_t>
typename sb_handle_t::event_t _reduction(sb_handle_t& sb, input_t buffer_in, index_t ld, output_t buffer_out,
                                         index_t rows, index_t cols, reduction_dim_t reduction_dim,
                                         const typename sb_handle_t::event_t& deps = {}) {
  sb.depend(deps);
  if constexpr (std::is_same_v<element_t, float>)
    return sb.done(gbblas_sreduction(sb.native(), operator_t::code, int(reduction_dim), buffer_in, ld, buffer_out,
                                     rows, cols));
  else if constexpr (std::is_same_v<element_t, double>)
    return sb.done(gbblas_dreduction(sb.native(), operator_t::code, int(reduction_dim), buffer_in, ld, buffer_out,
                                     rows, cols));
  else
    throw unsupported_exception("_reduction: element type not supported");
}
}  // namespace extension

}  // namespace blas

#endif  // PORTBLAS_GB_H

// gemm.cu — C ABI front end of the GEMM family: argument checks, the
// alpha == 0 shortcut, and method/tile selection.
//
// Follows internal::_gemm_backend (src/interface/gemm_interface.hpp:102-185):
//   - alpha == 0: C <- beta*C (zeros when beta == 0), A and B unread, and no
//     transpose validation (:112-139);
//   - trans is case-insensitive and must be n, t or c; c == t for real types
//     (:141-151);
//   - a strided batch with stride_c < ldc*n or any negative stride is
//     rejected (:153-166);
//   - _gemm_batched's default strides (:200-226).
#include <cctype>

#include "gemm_internal.cuh"
#include "selector.h"

namespace gb {

static bool parse_trans(char t, bool* tr) {
  const char l = char(std::tolower(static_cast<unsigned char>(t)));
  if (l == 'n') { *tr = false; return true; }
  if (l == 't' || l == 'c') { *tr = true; return true; }
  return false;
}

template <typename T>
static gbblas_status_t gemm_front(gbblas_handle_t h, char transa, char transb, int64_t m, int64_t n, int64_t k,
                                  T alpha, const T* a, int64_t lda, int64_t stride_a, const T* b, int64_t ldb,
                                  int64_t stride_b, T beta, T* c, int64_t ldc, int64_t stride_c, int64_t batch,
                                  bool strided_batch_checks) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "gemm: null handle");
  if (m < 0 || n < 0 || k < 0 || batch < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "gemm: negative dimension");
  if (m == 0 || n == 0 || batch == 0) return GBBLAS_STATUS_SUCCESS;
  if (!c) return fail(GBBLAS_STATUS_INVALID_ARG, "gemm: null C");
  if (alpha == T(0)) return launch_scale_c(h, m, n, beta, c, ldc, stride_c, batch);
  bool ta, tb;
  if (!parse_trans(transa, &ta)) return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _TransA");
  if (!parse_trans(transb, &tb)) return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _TransB");
  if (strided_batch_checks && batch > 1) {
    if (stride_c < ldc * n || stride_c < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _stridec");
    if (stride_a < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _stridea");
    if (stride_b < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _strideb");
  }
  if (k > 0 && (!a || !b)) return fail(GBBLAS_STATUS_INVALID_ARG, "gemm: null A or B");
  GemmArgs<T> g{ta, tb, m, n, k, alpha, beta, a, lda, stride_a, b, ldb, stride_b, c, ldc, stride_c, batch};
  return dispatch_gemm(h, g);
}

// FP64: the selector's pick among the FP64 SIMT configs (tile x split-K)
gbblas_status_t dispatch_gemm(gbblas_handle_t h, const GemmArgs<double>& g) {
  gbblas_status_t s = launch_dgemm_config(h, g, select_dgemm_config(h, g));
  if (s != GBBLAS_STATUS_UNSUPPORTED) return s;
  clear_error();  // a config that cannot take this shape (grid / workspace limits)
  return launch_gemm_simt(h, g);
}

gbblas_status_t dispatch_gemm(gbblas_handle_t h, const GemmArgs<float>& g) {
  switch (h->sgemm_mode) {
    case GBBLAS_SGEMM_FP32_SIMT: return launch_gemm_simt(h, g);
    case GBBLAS_SGEMM_SPLIT_BF16X3: return launch_gemm_split_bf16(h, g, 2);
    case GBBLAS_SGEMM_SPLIT_BF16X6: return launch_gemm_split_bf16(h, g, 3);
    default: break;
  }
  // AUTO: many small problems go to the one-CTA-per-problem kernel; shapes
  // that were not autotuned take the fixed x6 path (FP32-accurate) when they
  // are beyond the largest the selector was trained on (2 m n k batch > 2^35
  // flop: 8192^3 at 322 TFLOP/s against 236 for the selector's extrapolated
  // pick) or when they fit the 256 x 256 CTA-pair tiles, which the
  // selector's configs do not include (against its picks: 2048^3 219 / 185,
  // 4096^2 x 512 208 / 153, 8192^2 x 128 174 / 70, 1792^2 x 4096 185 / 153
  // TFLOP/s); otherwise every config is FP32-accurate and the selector
  // picks one
  if (small_batched_applies(g, h->sm_count)) return launch_gemm_small_batched(h, g);
  if ((2.0 * double(g.m) * double(g.n) * double(g.k) * double(g.batch) > double(int64_t(1) << 35) ||
       split_bf16_pair256_fits(g, h->sm_count)) &&
      !has_tuned_config(g))
    return launch_gemm_split_bf16(h, g, 3);
  gbblas_status_t s = launch_sgemm_config(h, g, select_sgemm_config(h, g));
  if (s != GBBLAS_STATUS_UNSUPPORTED) return s;
  clear_error();  // a config that cannot take this shape (grid / workspace limits)
  return launch_gemm_simt(h, g);
}

template <typename T>
gbblas_status_t batched_front(gbblas_handle_t h, char ta, char tb, int64_t m, int64_t n, int64_t k, T alpha,
                                     const T* a, int64_t lda, const T* b, int64_t ldb, T beta, T* c, int64_t ldc,
                                     int64_t batch, int batch_type) {
  if (batch_type == GBBLAS_BATCH_INTERLEAVED && batch > 1) {
    if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "gemm: null handle");
    if (m < 0 || n < 0 || k < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "gemm: negative dimension");
    if (m == 0 || n == 0) return GBBLAS_STATUS_SUCCESS;
    bool tra = false, trb = false;
    if (alpha != T(0)) {
      if (!parse_trans(ta, &tra)) return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _TransA");
      if (!parse_trans(tb, &trb)) return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _TransB");
      if (k > 0 && (!a || !b)) return fail(GBBLAS_STATUS_INVALID_ARG, "gemm: null A or B");
    }
    if (!c) return fail(GBBLAS_STATUS_INVALID_ARG, "gemm: null C");
    GemmArgs<T> g{tra, trb, m, n, k, alpha, beta, a, lda, 0, b, ldb, 0, c, ldc, 0, batch};
    return launch_gemm_interleaved(h, g);
  }
  if (batch_type != GBBLAS_BATCH_STRIDED && batch_type != GBBLAS_BATCH_INTERLEAVED)
    return fail(GBBLAS_STATUS_INVALID_ARG, "gemm_batched: unknown batch type");
  const bool tra = std::tolower(static_cast<unsigned char>(ta)) != 'n';
  const bool trb = std::tolower(static_cast<unsigned char>(tb)) != 'n';
  const int64_t sa = tra ? m * lda : k * lda;
  const int64_t sb = trb ? ldb * k : n * ldb;
  const int64_t sc = ldc * n;
  return gemm_front<T>(h, ta, tb, m, n, k, alpha, a, lda, sa, b, ldb, sb, beta, c, ldc, sc, batch, true);
}

}  // namespace gb

using namespace gb;

extern "C" {

gbblas_status_t gbblas_sgemm(gbblas_handle_t h, char ta, char tb, int64_t m, int64_t n, int64_t k, float alpha,
                             const float* a, int64_t lda, const float* b, int64_t ldb, float beta, float* c,
                             int64_t ldc) {
  clear_error();
  return gemm_front<float>(h, ta, tb, m, n, k, alpha, a, lda, 0, b, ldb, 0, beta, c, ldc, 0, 1, false);
}

gbblas_status_t gbblas_dgemm(gbblas_handle_t h, char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha,
                             const double* a, int64_t lda, const double* b, int64_t ldb, double beta, double* c,
                             int64_t ldc) {
  clear_error();
  return gemm_front<double>(h, ta, tb, m, n, k, alpha, a, lda, 0, b, ldb, 0, beta, c, ldc, 0, 1, false);
}

gbblas_status_t gbblas_sgemm_batched(gbblas_handle_t h, char ta, char tb, int64_t m, int64_t n, int64_t k,
                                     float alpha, const float* a, int64_t lda, const float* b, int64_t ldb,
                                     float beta, float* c, int64_t ldc, int64_t batch, int batch_type) {
  clear_error();
  return batched_front<float>(h, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, batch, batch_type);
}

gbblas_status_t gbblas_dgemm_batched(gbblas_handle_t h, char ta, char tb, int64_t m, int64_t n, int64_t k,
                                     double alpha, const double* a, int64_t lda, const double* b, int64_t ldb,
                                     double beta, double* c, int64_t ldc, int64_t batch, int batch_type) {
  clear_error();
  return batched_front<double>(h, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, batch, batch_type);
}

gbblas_status_t gbblas_sgemm_strided_batched(gbblas_handle_t h, char ta, char tb, int64_t m, int64_t n, int64_t k,
                                             float alpha, const float* a, int64_t lda, int64_t sa, const float* b,
                                             int64_t ldb, int64_t sb, float beta, float* c, int64_t ldc,
                                             int64_t sc, int64_t batch) {
  clear_error();
  return gemm_front<float>(h, ta, tb, m, n, k, alpha, a, lda, sa, b, ldb, sb, beta, c, ldc, sc, batch, true);
}

gbblas_status_t gbblas_dgemm_strided_batched(gbblas_handle_t h, char ta, char tb, int64_t m, int64_t n, int64_t k,
                                             double alpha, const double* a, int64_t lda, int64_t sa,
                                             const double* b, int64_t ldb, int64_t sb, double beta, double* c,
                                             int64_t ldc, int64_t sc, int64_t batch) {
  clear_error();
  return gemm_front<double>(h, ta, tb, m, n, k, alpha, a, lda, sa, b, ldb, sb, beta, c, ldc, sc, batch, true);
}

}  // extern "C"

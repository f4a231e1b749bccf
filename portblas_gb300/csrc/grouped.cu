// grouped.cu — grouped GEMM over uneven problems.
#include "gemm_internal.cuh"

using namespace gb;

extern "C" gbblas_status_t gbblas_gemm_grouped(gbblas_handle_t h, int dtype, int64_t count, const char* transa,
                                               const char* transb, const int64_t* m, const int64_t* n,
                                               const int64_t* k, const float* alpha, const void* const* a,
                                               const int64_t* lda, const void* const* b, const int64_t* ldb,
                                               const float* beta, float* const* c, const int64_t* ldc) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "gemm_grouped: null handle");
  if (dtype != GBBLAS_DTYPE_F32) return fail(GBBLAS_STATUS_UNSUPPORTED, "gemm_grouped: dtype not built yet");
  for (int64_t i = 0; i < count; ++i) {
    gbblas_status_t s = gbblas_sgemm(h, transa[i], transb[i], m[i], n[i], k[i], alpha[i],
                                     static_cast<const float*>(a[i]), lda[i], static_cast<const float*>(b[i]),
                                     ldb[i], beta[i], c[i], ldc[i]);
    if (s != GBBLAS_STATUS_SUCCESS) return s;
  }
  return GBBLAS_STATUS_SUCCESS;
}

// gemm_tc.cu — split-BF16 FP32 GEMM on the tcgen05 tensor cores.
#include "gemm_internal.cuh"
#include "selector.h"

namespace gb {

gbblas_status_t launch_gemm_split_bf16(gbblas_handle_t, const GemmArgs<float>&, int) {
  return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: not built yet");
}

int select_sgemm_method(gbblas_handle_t, const GemmArgs<float>&) { return GBBLAS_SGEMM_FP32_SIMT; }

}  // namespace gb

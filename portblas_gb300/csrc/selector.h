// selector.h — choice of the FP32 GEMM method for GBBLAS_SGEMM_AUTO.
#pragma once
#include "gemm_internal.cuh"

namespace gb {

// Method for an FP32 GEMM under AUTO: the 3-way BF16 split (FP32-accurate)
// on the tensor cores once the problem is large enough to amortise the
// operand split, else the SIMT kernel.
int select_sgemm_method(gbblas_handle_t h, const GemmArgs<float>& g);

}  // namespace gb

// selector.h — FP32 GEMM configuration space and its selectors (selector.cu).
#pragma once
#include "gemm_internal.cuh"

namespace gb {

constexpr int kSgemmConfigs = 40;   // tile configurations of the FP32 GEMM
constexpr int kSgemmFeatures = 11;  // selector input features

// Runs config `config` (0..39) on the problem.
gbblas_status_t launch_sgemm_config(gbblas_handle_t h, const GemmArgs<float>& g, int config);

// Config for GBBLAS_SGEMM_AUTO: an autotuned winner for this shape if there
// is one, else the learned selector when its weights are loaded, else the
// fixed size-threshold heuristic.
int select_sgemm_config(gbblas_handle_t h, const GemmArgs<float>& g);

// The fixed size-threshold heuristic alone.
int heuristic_config(int64_t m, int64_t n, int64_t batch);

// Selector input features of a problem (kSgemmFeatures floats).
void sgemm_features(int64_t m, int64_t n, int64_t k, int ta, int tb, int64_t lda, int64_t ldb, int64_t ldc,
                    int64_t batch, float* f);

}  // namespace gb

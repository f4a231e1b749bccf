// selector.h — GEMM tile configuration space and its selectors (selector.cu).
#pragma once
#include "gemm_internal.cuh"

namespace gb {

// Configurations of the GEMM: 0..39 FP32 (SIMT tiles x split-K, split-BF16
// tcgen05 tiles x split-K x raster), 40..59 FP64 (SIMT tiles x split-K).
constexpr int kSgemmConfigs = 40;                  // FP32 configs: [0, 40)
constexpr int kDgemmFirst = 40, kDgemmConfigs = 20;  // FP64 configs: [40, 60)
constexpr int kGemmConfigs = kDgemmFirst + kDgemmConfigs;
constexpr int kSgemmFeatures = 11;  // selector input features

// Element type of a selector query: FP32 or FP64 (one-hot feature 9 / 10).
enum : int { kSelF32 = 0, kSelF64 = 1 };

// Runs FP32 config `config` (0..39) / FP64 config (40..59) on the problem.
gbblas_status_t launch_sgemm_config(gbblas_handle_t h, const GemmArgs<float>& g, int config);
gbblas_status_t launch_dgemm_config(gbblas_handle_t h, const GemmArgs<double>& g, int config);

// Config for AUTO: an autotuned winner for this shape if there is one, else
// the learned selector when its weights are loaded, else the fixed
// size-threshold heuristic; always one of the element type's configs.
int select_sgemm_config(gbblas_handle_t h, const GemmArgs<float>& g);
bool has_tuned_config(const GemmArgs<float>& g);  // an autotuned winner is stored for this shape
int select_dgemm_config(gbblas_handle_t h, const GemmArgs<double>& g);

// The fixed size-threshold heuristic alone.
int heuristic_config(int64_t m, int64_t n, int64_t batch, int dtype);

// Selector input features of a problem (kSgemmFeatures floats).
void gemm_features(int64_t m, int64_t n, int64_t k, int ta, int tb, int64_t lda, int64_t ldb, int64_t ldc,
                   int64_t batch, int dtype, float* f);

}  // namespace gb

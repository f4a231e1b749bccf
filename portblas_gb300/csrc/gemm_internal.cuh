// gemm_internal.cuh — internal launch interface of the GEMM kernels.
#pragma once
#include "common.cuh"

namespace gb {

// One (possibly batched) column-major GEMM problem.  Element (i, j) of op(A)
// is A[i + j*lda] (ta false) or A[j + i*lda] (ta true); same for B.
template <typename T>
struct GemmArgs {
  bool ta, tb;
  int64_t m, n, k;
  T alpha, beta;
  const T* a;
  int64_t lda, stride_a;
  const T* b;
  int64_t ldb, stride_b;
  T* c;
  int64_t ldc, stride_c;
  int64_t batch;
};

// Plain FP32 / FP64 SIMT GEMM (CUDA cores), any transposes, strided batch.
gbblas_status_t launch_gemm_simt(gbblas_handle_t h, const GemmArgs<float>& g);
// Interleaved batch (batch fastest): element (r, c) of matrix b at
// ptr[(r + c*ld)*batch + b].
gbblas_status_t launch_gemm_interleaved(gbblas_handle_t h, const GemmArgs<float>& g);
gbblas_status_t launch_gemm_interleaved(gbblas_handle_t h, const GemmArgs<double>& g);
// Strided batches of small FP32 problems (M, N, K <= 64, batch >= 4 per SM):
// one CTA per problem.
bool small_batched_applies(const GemmArgs<float>& g, int sm_count);
gbblas_status_t launch_gemm_small_batched(gbblas_handle_t h, const GemmArgs<float>& g);
// The same batches (M, N, K <= 64) on the tcgen05 tensor cores, two problems
// per tile; UNSUPPORTED (nothing launched) when TMA cannot address the layout.
gbblas_status_t launch_gemm_small_batched_tc(gbblas_handle_t h, const GemmArgs<float>& g);
// FP32 / FP64 SIMT GEMM with an explicit CTA tile and split-K factor.
enum : int { kSimtTile128x128 = 0, kSimtTile128x64 = 1, kSimtTile64x128 = 2, kSimtTile64x64 = 3 };
gbblas_status_t launch_gemm_simt_tiled(gbblas_handle_t h, const GemmArgs<float>& g, int tile, int split);
gbblas_status_t launch_gemm_simt_tiled(gbblas_handle_t h, const GemmArgs<double>& g, int tile, int split);
gbblas_status_t launch_gemm_simt(gbblas_handle_t h, const GemmArgs<double>& g);

// C <- beta*C over a strided batch of M x N matrices (beta == 0 writes zeros):
// the alpha == 0 path of gemm_interface.hpp:112-139.
gbblas_status_t launch_scale_c(gbblas_handle_t h, int64_t m, int64_t n, float beta, float* c, int64_t ldc,
                               int64_t stride_c, int64_t batch);
gbblas_status_t launch_scale_c(gbblas_handle_t h, int64_t m, int64_t n, double beta, double* c, int64_t ldc,
                               int64_t stride_c, int64_t batch);

// Split-BF16 FP32 GEMM on the tcgen05 tensor cores (pieces = 2 or 3 BF16
// terms per operand).  Returns UNSUPPORTED when the shape is not handled.
gbblas_status_t launch_gemm_split_bf16(gbblas_handle_t h, const GemmArgs<float>& g, int pieces);
// The fixed split-BF16 modes take 256 x 256 CTA-pair tiles for this shape
// (M and N at least 256, enough tiles, the last round filled well enough).
bool split_bf16_pair256_fits(const GemmArgs<float>& g, int64_t sm_count);
// The tiles launch_gemm_split_bf16 runs this shape on (pieces: 2 = x3,
// 3 = x6): output tile tile_m x tile_n (tile_m 256: a CTA pair) and the
// number of split-K slices.
struct SplitBf16Route {
  int tile_m, tile_n, k_slices;
};
SplitBf16Route split_bf16_route(const GemmArgs<float>& g, int pieces, int64_t sm_count);
// Same with an explicit N tile (64 or 128), split-K factor and raster order
// (raster_m: consecutive CTAs walk down M).
gbblas_status_t launch_gemm_split_bf16_cfg(gbblas_handle_t h, const GemmArgs<float>& g, int pieces, int bn,
                                           int split, int raster_m);

// Sums split-K partial tiles ws[batch][split][M][N] in slice order into C
// with the alpha/beta epilogue (deterministic).
gbblas_status_t launch_splitk_reduce(gbblas_handle_t h, const GemmArgs<float>& g, int split, const float* ws);

// Method dispatch after argument checks (gemm.cu).
gbblas_status_t dispatch_gemm(gbblas_handle_t h, const GemmArgs<float>& g);
gbblas_status_t dispatch_gemm(gbblas_handle_t h, const GemmArgs<double>& g);

}  // namespace gb

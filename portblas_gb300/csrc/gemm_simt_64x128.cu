// gemm_simt_64x128.cu — SIMT GEMM kernels with a 64x128 CTA tile (one
// translation unit per tile so the library compiles in parallel).
#include "gemm_simt.cuh"

namespace gb {

gbblas_status_t launch_simt_tile_64x128(gbblas_handle_t h, const GemmArgs<float>& g, int split) {
  return launch_simt_cfg<float, 64, 128, 4, 8>(h, g, split);
}

gbblas_status_t launch_simt_tile_64x128_f64(gbblas_handle_t h, const GemmArgs<double>& g, int split) {
  return launch_simt_cfg<double, 64, 128, 4, 8>(h, g, split);
}

}  // namespace gb

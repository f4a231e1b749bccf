// gemm_simt_128x128.cu — SIMT GEMM kernels with a 128x128 CTA tile (one
// translation unit per tile so the library compiles in parallel).
#include "gemm_simt.cuh"

namespace gb {

gbblas_status_t launch_simt_tile_128x128(gbblas_handle_t h, const GemmArgs<float>& g, int split) {
  return launch_simt_cfg<float, 128, 128, 8, 8>(h, g, split);
}

gbblas_status_t launch_simt_tile_128x128_f64(gbblas_handle_t h, const GemmArgs<double>& g, int split) {
  return launch_simt_cfg<double, 128, 128, 8, 8>(h, g, split);
}

}  // namespace gb

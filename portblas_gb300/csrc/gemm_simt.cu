// gemm_simt.cu — dispatch of the SIMT GEMM tiles (kernels in gemm_simt.cuh,
// one translation unit per tile), the split-K reduction, the interleaved
// batch kernel and the alpha == 0 scaling of C.
#include "gemm_simt.cuh"

namespace gb {

gbblas_status_t launch_splitk_reduce(gbblas_handle_t h, const GemmArgs<float>& g, int split, const float* ws) {
  const int64_t total = g.m * g.n * g.batch;
  const int64_t blocks = cdiv(total, 256) < int64_t(h->sm_count) * 8 ? cdiv(total, 256) : int64_t(h->sm_count) * 8;
  splitk_reduce_kernel<float><<<unsigned(blocks), 256, 0, h->stream>>>(g, split, ws, g.batch);
  return after_launch("splitk_reduce");
}

gbblas_status_t launch_simt_tile_128x128(gbblas_handle_t h, const GemmArgs<float>& g, int split);
gbblas_status_t launch_simt_tile_128x64(gbblas_handle_t h, const GemmArgs<float>& g, int split);
gbblas_status_t launch_simt_tile_64x128(gbblas_handle_t h, const GemmArgs<float>& g, int split);
gbblas_status_t launch_simt_tile_64x64(gbblas_handle_t h, const GemmArgs<float>& g, int split);
gbblas_status_t launch_simt_tile_128x128_f64(gbblas_handle_t h, const GemmArgs<double>& g, int split);

gbblas_status_t launch_gemm_simt_tiled(gbblas_handle_t h, const GemmArgs<float>& g, int tile, int split) {
  switch (tile) {
    case kSimtTile128x128: return launch_simt_tile_128x128(h, g, split);
    case kSimtTile128x64: return launch_simt_tile_128x64(h, g, split);
    case kSimtTile64x128: return launch_simt_tile_64x128(h, g, split);
    case kSimtTile64x64: return launch_simt_tile_64x64(h, g, split);
  }
  return fail(GBBLAS_STATUS_INVALID_ARG, "gemm: unknown SIMT tile");
}

gbblas_status_t launch_gemm_simt(gbblas_handle_t h, const GemmArgs<float>& g) {
  return launch_simt_tile_128x128(h, g, 1);
}
gbblas_status_t launch_gemm_simt(gbblas_handle_t h, const GemmArgs<double>& g) {
  return launch_simt_tile_128x128_f64(h, g, 1);
}

// ------------------------------------------------------ small batches --
// Strided batches of small problems (M, N, K <= 64): one CTA per problem
// loads all of A and B into shared memory in one coalesced pass (a single
// wait instead of one per k-slab), each of 256 threads computes a 4x4 block,
// and C goes back through shared memory so the stores are coalesced too.
constexpr int kSmallMax = 64;

template <bool TA, bool TB>
__global__ void __launch_bounds__(256) gemm_small_batched_kernel(GemmArgs<float> g) {
  __shared__ float As[kSmallMax][kSmallMax + 4];  // [k][i]
  __shared__ float Bs[kSmallMax][kSmallMax + 4];  // [k][j]
  const int64_t bz = blockIdx.x;
  const float* A = g.a + bz * g.stride_a;
  const float* B = g.b + bz * g.stride_b;
  float* C = g.c + bz * g.stride_c;
  const int M = int(g.m), N = int(g.n), K = int(g.k), t = threadIdx.x;
  for (int e = t; e < M * K; e += 256) {
    int i, k;
    if (!TA) { i = e % M; k = e / M; } else { k = e % K; i = e / K; }
    As[k][i] = TA ? A[k + int64_t(i) * g.lda] : A[i + int64_t(k) * g.lda];
  }
  for (int e = t; e < K * N; e += 256) {
    int k, j;
    if (!TB) { k = e % K; j = e / K; } else { j = e % N; k = e / N; }
    Bs[k][j] = TB ? B[j + int64_t(k) * g.ldb] : B[k + int64_t(j) * g.ldb];
  }
  __syncthreads();
  const int tx = t % 16, ty = t / 16;
  float acc[4][4] = {};
  for (int k = 0; k < K; ++k) {
    float a[4], b[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      a[q] = As[k][ty * 4 + q];
      b[q] = Bs[k][tx * 4 + q];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
  }
  __syncthreads();
  // stage C in As as [j][i] for coalesced column-major stores
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) As[tx * 4 + j][ty * 4 + i] = acc[i][j];
  __syncthreads();
  for (int e = t; e < M * N; e += 256) {
    const int i = e % M, j = e / M;
    float* cp = C + i + int64_t(j) * g.ldc;
    float v = g.alpha * As[j][i];
    if (g.beta != 0.f) v = fmaf(g.beta, *cp, v);
    *cp = v;
  }
}

bool small_batched_applies(const GemmArgs<float>& g, int sm_count) {
  return g.m <= kSmallMax && g.n <= kSmallMax && g.k <= kSmallMax && g.batch >= 4 * int64_t(sm_count) &&
         g.batch <= INT32_MAX;
}

gbblas_status_t launch_gemm_small_batched(gbblas_handle_t h, const GemmArgs<float>& g) {
  const dim3 grid(unsigned(g.batch));
#define GB_SMALL(TA_, TB_) \
  if (g.ta == TA_ && g.tb == TB_) gemm_small_batched_kernel<TA_, TB_><<<grid, 256, 0, h->stream>>>(g);
  GB_SMALL(false, false)
  GB_SMALL(false, true)
  GB_SMALL(true, false)
  GB_SMALL(true, true)
#undef GB_SMALL
  return after_launch("gemm_small_batched");
}

// ----------------------------------------------------------- interleaved --
// gemm_batch_type_t::interleaved (src/operations/blas3/gemm_interleaved.hpp,
// layout as in test/unittest/blas3/blas3_gemm_common.hpp:53-87): the batch
// is the fastest axis, element (r, c) of matrix b of an operand with leading
// dimension ld is at ptr[(r + c*ld)*batch + b].  Consecutive threads take
// consecutive batch entries, so every load and store is coalesced; each
// thread accumulates a 4x4 block of its own problem's C.
template <typename T>
__global__ void __launch_bounds__(128) gemm_interleaved_kernel(GemmArgs<T> g) {
  constexpr int TI = 4, TJ = 4;
  const int64_t b = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (b >= g.batch) return;
  const int64_t tiles_i = (g.m + TI - 1) / TI;
  const int64_t i0 = (int64_t(blockIdx.y) % tiles_i) * TI, j0 = (int64_t(blockIdx.y) / tiles_i) * TJ;
  const int64_t B = g.batch;
  T acc[TI][TJ];
#pragma unroll
  for (int i = 0; i < TI; ++i)
#pragma unroll
    for (int j = 0; j < TJ; ++j) acc[i][j] = T(0);
  if (g.alpha != T(0)) {
    for (int64_t k = 0; k < g.k; ++k) {
      T av[TI], bv[TJ];
#pragma unroll
      for (int i = 0; i < TI; ++i) {
        const int64_t gi = i0 + i;
        av[i] = gi < g.m ? g.a[((g.ta ? k + gi * g.lda : gi + k * g.lda)) * B + b] : T(0);
      }
#pragma unroll
      for (int j = 0; j < TJ; ++j) {
        const int64_t gj = j0 + j;
        bv[j] = gj < g.n ? g.b[((g.tb ? gj + k * g.ldb : k + gj * g.ldb)) * B + b] : T(0);
      }
#pragma unroll
      for (int i = 0; i < TI; ++i)
#pragma unroll
        for (int j = 0; j < TJ; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
  }
#pragma unroll
  for (int j = 0; j < TJ; ++j) {
    const int64_t gj = j0 + j;
    if (gj >= g.n) continue;
#pragma unroll
    for (int i = 0; i < TI; ++i) {
      const int64_t gi = i0 + i;
      if (gi >= g.m) continue;
      T* cp = g.c + (gi + gj * g.ldc) * B + b;
      T r = g.alpha * acc[i][j];
      if (g.beta != T(0)) r = fma(g.beta, *cp, r);
      else if (g.alpha == T(0)) r = T(0);
      *cp = r;
    }
  }
}

template <typename T>
gbblas_status_t interleaved_impl(gbblas_handle_t h, const GemmArgs<T>& g) {
  const int64_t tiles = ((g.m + 3) / 4) * ((g.n + 3) / 4);
  if (tiles > 65535) return fail(GBBLAS_STATUS_UNSUPPORTED, "gemm_batched interleaved: matrices too large");
  dim3 grid(unsigned(cdiv(g.batch, 128)), unsigned(tiles));
  gemm_interleaved_kernel<T><<<grid, 128, 0, h->stream>>>(g);
  return after_launch("gemm_interleaved");
}

gbblas_status_t launch_gemm_interleaved(gbblas_handle_t h, const GemmArgs<float>& g) { return interleaved_impl(h, g); }
gbblas_status_t launch_gemm_interleaved(gbblas_handle_t h, const GemmArgs<double>& g) {
  return interleaved_impl(h, g);
}

// ------------------------------------------------------------- scale C --
template <typename T>
__global__ void scale_c_kernel(int64_t m, int64_t n, T beta, T* c, int64_t ldc, int64_t stride_c) {
  T* C = c + int64_t(blockIdx.z) * stride_c;
  const int64_t j = int64_t(blockIdx.y);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < m; i += int64_t(gridDim.x) * blockDim.x) {
    T* p = C + i + j * ldc;
    *p = beta == T(0) ? T(0) : beta * *p;  // scal by 0 writes zeros (blas1_interface.hpp:438-455)
  }
}

template <typename T>
gbblas_status_t scale_c_impl(gbblas_handle_t h, int64_t m, int64_t n, T beta, T* c, int64_t ldc, int64_t stride_c,
                             int64_t batch) {
  if (m <= 0 || n <= 0 || batch <= 0) return GBBLAS_STATUS_SUCCESS;
  for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
    const int64_t nb = batch - b0 < 65535 ? batch - b0 : 65535;
    for (int64_t j0 = 0; j0 < n; j0 += 65535) {
      const int64_t nj = n - j0 < 65535 ? n - j0 : 65535;
      dim3 grid(unsigned(cdiv(m, 256) < 64 ? cdiv(m, 256) : 64), unsigned(nj), unsigned(nb));
      scale_c_kernel<T><<<grid, 256, 0, h->stream>>>(m, nj, beta, c + b0 * stride_c + j0 * ldc, ldc, stride_c);
      GB_TRY(after_launch("scale_c"));
    }
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t launch_scale_c(gbblas_handle_t h, int64_t m, int64_t n, float beta, float* c, int64_t ldc,
                               int64_t stride_c, int64_t batch) {
  return scale_c_impl(h, m, n, beta, c, ldc, stride_c, batch);
}
gbblas_status_t launch_scale_c(gbblas_handle_t h, int64_t m, int64_t n, double beta, double* c, int64_t ldc,
                               int64_t stride_c, int64_t batch) {
  return scale_c_impl(h, m, n, beta, c, ldc, stride_c, batch);
}

}  // namespace gb

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
gbblas_status_t launch_simt_tile_128x64_f64(gbblas_handle_t h, const GemmArgs<double>& g, int split);
gbblas_status_t launch_simt_tile_64x128_f64(gbblas_handle_t h, const GemmArgs<double>& g, int split);
gbblas_status_t launch_simt_tile_64x64_f64(gbblas_handle_t h, const GemmArgs<double>& g, int split);

gbblas_status_t launch_gemm_simt_tiled(gbblas_handle_t h, const GemmArgs<float>& g, int tile, int split) {
  switch (tile) {
    case kSimtTile128x128: return launch_simt_tile_128x128(h, g, split);
    case kSimtTile128x64: return launch_simt_tile_128x64(h, g, split);
    case kSimtTile64x128: return launch_simt_tile_64x128(h, g, split);
    case kSimtTile64x64: return launch_simt_tile_64x64(h, g, split);
  }
  return fail(GBBLAS_STATUS_INVALID_ARG, "gemm: unknown SIMT tile");
}

gbblas_status_t launch_gemm_simt_tiled(gbblas_handle_t h, const GemmArgs<double>& g, int tile, int split) {
  switch (tile) {
    case kSimtTile128x128: return launch_simt_tile_128x128_f64(h, g, split);
    case kSimtTile128x64: return launch_simt_tile_128x64_f64(h, g, split);
    case kSimtTile64x128: return launch_simt_tile_64x128_f64(h, g, split);
    case kSimtTile64x64: return launch_simt_tile_64x64_f64(h, g, split);
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
// loads all of A and B into shared memory in one coalesced pass (128-bit
// loads along the contiguous dimension when it is 16-byte aligned), each of
// 256 threads computes a 4x4 block from 128-bit shared reads, and C goes
// back through shared memory so the stores are coalesced too.
constexpr int kSmallMax = 64;

// S[k][r] <- X(r, k) for r < R, k < K, X(r, k) = X[r*sr + k*sk] with one of
// sr, sk equal to 1 (RC: rows contiguous).  Thread t takes vector t % 16 of
// the contiguous dimension and strides the other by 16.
template <bool RC>
__device__ __forceinline__ void small_stage(float (&S)[kSmallMax][kSmallMax + 4], const float* __restrict__ X,
                                            int64_t ld, int R, int K, int t) {
  const int v = t & 15, o = t >> 4;
  const int C = RC ? R : K;  // contiguous extent
  const int O = RC ? K : R;  // other extent
  const bool vec = (C & 3) == 0 && (ld & 3) == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0;
  if (vec) {
    if (4 * v < C)
      for (int q = o; q < O; q += 16) {
        const float4 x = __ldg(reinterpret_cast<const float4*>(X + int64_t(q) * ld) + v);
        if (RC) {  // rows contiguous: S[q][4v..4v+3]
          *reinterpret_cast<float4*>(&S[q][4 * v]) = x;
        } else {  // k contiguous: S[4v..4v+3][q]
          S[4 * v][q] = x.x;
          S[4 * v + 1][q] = x.y;
          S[4 * v + 2][q] = x.z;
          S[4 * v + 3][q] = x.w;
        }
      }
    return;
  }
  for (int q = o; q < O; q += 16)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int c = 4 * v + e;
      if (c < C) {
        const float x = __ldg(X + int64_t(q) * ld + c);
        if (RC) S[q][c] = x;
        else S[c][q] = x;
      }
    }
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(256, 6) gemm_small_batched_kernel(GemmArgs<float> g) {
  __shared__ __align__(16) float As[kSmallMax][kSmallMax + 4];  // [k][i]
  __shared__ __align__(16) float Bs[kSmallMax][kSmallMax + 4];  // [k][j]
  const int64_t bz = blockIdx.x;
  const float* A = g.a + bz * g.stride_a;
  const float* B = g.b + bz * g.stride_b;
  float* C = g.c + bz * g.stride_c;
  const int M = int(g.m), N = int(g.n), K = int(g.k), t = threadIdx.x;
  // A(i, k) = TA ? A[k + i*lda] : A[i + k*lda];  B(k, j) = TB ? B[j + k*ldb] : B[k + j*ldb]
  small_stage<!TA>(As, A, g.lda, M, K, t);
  small_stage<TB>(Bs, B, g.ldb, N, K, t);
  __syncthreads();
  const int tx = t % 16, ty = t / 16;
  float acc[4][4] = {};
  for (int k = 0; k < K; ++k) {
    const float4 a = *reinterpret_cast<const float4*>(&As[k][ty * 4]);
    const float4 b = *reinterpret_cast<const float4*>(&Bs[k][tx * 4]);
#define GB_ROW(i, ai)                         \
  acc[i][0] = fmaf(ai, b.x, acc[i][0]);       \
  acc[i][1] = fmaf(ai, b.y, acc[i][1]);       \
  acc[i][2] = fmaf(ai, b.z, acc[i][2]);       \
  acc[i][3] = fmaf(ai, b.w, acc[i][3]);
    GB_ROW(0, a.x)
    GB_ROW(1, a.y)
    GB_ROW(2, a.z)
    GB_ROW(3, a.w)
#undef GB_ROW
  }
  __syncthreads();
  // stage C in As as [j][i] for coalesced column-major stores
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) As[tx * 4 + j][ty * 4 + i] = acc[i][j];
  __syncthreads();
  const int i = t & 63;
  if (i < M)
    for (int j = t >> 6; j < N; j += 4) {
      float* cp = C + i + int64_t(j) * g.ldc;
      float v = g.alpha * As[j][i];
      if (g.beta != 0.f) v = fmaf(g.beta, *cp, v);
      *cp = v;
    }
}

// ------------------------------------------- small batches, 8 x 8 tiles --
// The 16-byte-aligned case (M, N, K multiples of 4, leading dimensions and
// strides multiples of 4 floats): persistent 64-thread CTAs, six per SM,
// walk the batch one problem at a time.  A CTA copies the problem's A and B
// into shared memory with 16-byte cp.async (memory layout kept: 64 rows of
// 64 floats; rows whose k is contiguous have their 16-byte chunks XOR-
// swizzled by row / 8), then each thread computes an 8 x 8 block of C from
// 128-bit shared reads: 4 k at a time, 8 + 8 reads feed 256 FMAs, and every
// read of a warp is conflict-free (its rows share one swizzle key per
// thread and differ across threads).  While one CTA computes, the others on
// its SM wait on their copies, so the copies and the FMAs overlap.  (Six
// single-buffered CTAs measured faster than three double-buffered ones:
// 64.5 against 75.6 us for 4096 x 64^3; the earlier 4 x 4 tiles ran 73 us.)
constexpr int kR8Threads = 64;
constexpr int kR8CtasPerSm = 6;
constexpr int kR8Row = 64;                          // floats per shared row
constexpr int kR8Tile = kSmallMax * kR8Row;         // floats per operand

__device__ __forceinline__ int r8_swz(int row, int chunk) { return (chunk ^ ((row >> 3) & 7)) * 4; }

__device__ __forceinline__ void cp_async16(float* dst, const float* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(dst))),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// rows x cols floats of X (row r at X + r*ld, cols contiguous) into S;
// SWZ: chunk c of row r goes to chunk c ^ ((r / 8) % 8)
template <bool SWZ>
__device__ __forceinline__ void r8_copy(float* S, const float* X, int64_t ld, int rows, int cols, int t) {
  const int cpr = cols >> 2;  // chunks per row
  for (int e = t; e < rows * 16; e += kR8Threads) {
    const int r = e >> 4, c = e & 15;
    if (c < cpr) cp_async16(S + r * kR8Row + (SWZ ? r8_swz(r, c) : 4 * c), X + int64_t(r) * ld + 4 * c);
  }
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(kR8Threads, kR8CtasPerSm) gemm_small_batched_r8_kernel(GemmArgs<float> g) {
  extern __shared__ __align__(16) float r8_smem[];  // [A, B][kR8Tile]
  float* SA = r8_smem;
  float* SB = r8_smem + kR8Tile;
  const int M = int(g.m), N = int(g.n), K = int(g.k), t = threadIdx.x;
  const int tx = t & 7, ty = t >> 3;  // C rows 8ty .. 8ty+7, columns 8tx .. 8tx+7
  // A(i, k): TA ? rows i, k contiguous (swizzled) : rows k, i contiguous
  // B(k, j): TB ? rows k, j contiguous : rows j, k contiguous (swizzled)
  for (int64_t p = blockIdx.x; p < g.batch; p += gridDim.x) {
    const float* A = g.a + p * g.stride_a;
    const float* B = g.b + p * g.stride_b;
    if (TA) r8_copy<true>(SA, A, g.lda, M, K, t);
    else r8_copy<false>(SA, A, g.lda, K, M, t);
    if (TB) r8_copy<false>(SB, B, g.ldb, K, N, t);
    else r8_copy<true>(SB, B, g.ldb, N, K, t);
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
#pragma unroll 2
    for (int k = 0; k < K; k += 4) {
      float a[8][4], b[4][8];  // a[i][kk] = A(8ty+i, k+kk), b[kk][j] = B(k+kk, 8tx+j)
      if (TA) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const float4 v = *reinterpret_cast<const float4*>(SA + (8 * ty + i) * kR8Row + r8_swz(8 * ty, k >> 2));
          a[i][0] = v.x; a[i][1] = v.y; a[i][2] = v.z; a[i][3] = v.w;
        }
      } else {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float4 v = *reinterpret_cast<const float4*>(SA + (k + kk) * kR8Row + 8 * ty + 4 * h);
            a[4 * h][kk] = v.x; a[4 * h + 1][kk] = v.y; a[4 * h + 2][kk] = v.z; a[4 * h + 3][kk] = v.w;
          }
      }
      if (TB) {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float4 v = *reinterpret_cast<const float4*>(SB + (k + kk) * kR8Row + 8 * tx + 4 * h);
            b[kk][4 * h] = v.x; b[kk][4 * h + 1] = v.y; b[kk][4 * h + 2] = v.z; b[kk][4 * h + 3] = v.w;
          }
      } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float4 v = *reinterpret_cast<const float4*>(SB + (8 * tx + j) * kR8Row + r8_swz(8 * tx, k >> 2));
          b[0][j] = v.x; b[1][j] = v.y; b[2][j] = v.z; b[3][j] = v.w;
        }
      }
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i][kk], b[kk][j], acc[i][j]);
    }
    __syncthreads();  // the operands of the next problem overwrite these buffers
    // C(i, j), i = 8ty.., j = 8tx..: each column's 8 rows as two 128-bit
    // accesses; a column's old values are loaded before its stores
    float* C = g.c + p * g.stride_c;
    if (8 * ty < M) {
      const bool two = 8 * ty + 4 < M;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int gj = 8 * tx + j;
        if (gj >= N) continue;
        float4* cp = reinterpret_cast<float4*>(C + 8 * ty + int64_t(gj) * g.ldc);
        float4 v0 = make_float4(g.alpha * acc[0][j], g.alpha * acc[1][j], g.alpha * acc[2][j], g.alpha * acc[3][j]);
        float4 v1 = make_float4(g.alpha * acc[4][j], g.alpha * acc[5][j], g.alpha * acc[6][j], g.alpha * acc[7][j]);
        if (g.beta != 0.f) {
          const float4 o0 = cp[0];
          const float4 o1 = two ? cp[1] : make_float4(0.f, 0.f, 0.f, 0.f);
          v0.x = fmaf(g.beta, o0.x, v0.x); v0.y = fmaf(g.beta, o0.y, v0.y);
          v0.z = fmaf(g.beta, o0.z, v0.z); v0.w = fmaf(g.beta, o0.w, v0.w);
          v1.x = fmaf(g.beta, o1.x, v1.x); v1.y = fmaf(g.beta, o1.y, v1.y);
          v1.z = fmaf(g.beta, o1.z, v1.z); v1.w = fmaf(g.beta, o1.w, v1.w);
        }
        cp[0] = v0;
        if (two) cp[1] = v1;
      }
    }
  }
}

static bool small_pipe_applies(const GemmArgs<float>& g) {
  auto a16 = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15) == 0; };
  return g.m % 4 == 0 && g.n % 4 == 0 && g.k % 4 == 0 && g.k > 0 && g.lda % 4 == 0 && g.ldb % 4 == 0 &&
         g.ldc % 4 == 0 && g.stride_a % 4 == 0 && g.stride_b % 4 == 0 && g.stride_c % 4 == 0 && a16(g.a) &&
         a16(g.b) && a16(g.c) && g.alpha != 0.f;
}

bool small_batched_applies(const GemmArgs<float>& g, int sm_count) {
  return g.m <= kSmallMax && g.n <= kSmallMax && g.k <= kSmallMax && g.batch >= 4 * int64_t(sm_count) &&
         g.batch <= INT32_MAX;
}

gbblas_status_t launch_gemm_small_batched(gbblas_handle_t h, const GemmArgs<float>& g) {
  {
    const gbblas_status_t s = launch_gemm_small_batched_tc(h, g);
    if (s != GBBLAS_STATUS_UNSUPPORTED) return s;
  }
  if (small_pipe_applies(g)) {
    constexpr int smem = 2 * kR8Tile * int(sizeof(float));
    const int64_t cap = int64_t(h->sm_count) * kR8CtasPerSm;
    const unsigned grid = unsigned(g.batch < cap ? g.batch : cap);
#define GB_R8(TA_, TB_)                                                                                     \
  if (g.ta == TA_ && g.tb == TB_) {                                                                         \
    static std::atomic<uint64_t> attr{0};                                                                   \
    GB_CUDA_TRY(raise_smem_limit(attr, reinterpret_cast<const void*>(gemm_small_batched_r8_kernel<TA_, TB_>), \
                                 smem, h->device));                                                         \
    gemm_small_batched_r8_kernel<TA_, TB_><<<grid, kR8Threads, smem, h->stream>>>(g);                        \
  }
    GB_R8(false, false)
    GB_R8(false, true)
    GB_R8(true, false)
    GB_R8(true, true)
#undef GB_R8
    return after_launch("gemm_small_batched_r8");
  }
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

// gemm_simt.cu — plain FP32 / FP64 GEMM on the CUDA cores (SIMT FMA).
//
// This is the "plain FP32" comparator of the split-BF16 tensor-core SGEMM and
// the FP64-pipe DGEMM.  It plays the role of portBLAS's Gemm<local, ...>
// kernel (src/operations/blas3/gemm_local.hpp:74-875), which stages A and B
// blocks in work-group local memory and accumulates a register tile with
// sycl::mad; the structure here is the usual CUDA one: a 128x128 CTA tile,
// k-major shared-memory stages filled from registers (so any transpose is a
// register shuffle), an 8x8 register micro-tile per thread split into four
// 4x4 quadrants 64 apart (conflict-free 128-bit shared loads), double
// buffering, and a fused alpha/beta epilogue.  The epilogue is
// alpha*acc + beta*C (gemm_ref.hpp:240-250); beta == 0 never reads C
// (gemm_local.hpp:401-409).  Strided batches run on gridDim.z.
#include "gemm_internal.cuh"

namespace gb {

template <typename T>
struct SimtCfg;
template <>
struct SimtCfg<float> {
  static constexpr int BK = 16;
};
template <>
struct SimtCfg<double> {
  static constexpr int BK = 8;
};

template <typename T>
struct VecT;
template <>
struct VecT<float> {
  using V = float4;
  static constexpr int W = 4;
};
template <>
struct VecT<double> {
  using V = double2;
  static constexpr int W = 2;
};

constexpr int kBM = 128, kBN = 128, kSimtThreads = 256;

// Loads one BK-deep slab of an operand tile into registers.  Element (r, k)
// of the slab (r along M or N, k along K) lives at src[r + k*ld] when
// R_CONTIG (r contiguous) and at src[k + r*ld] otherwise.
template <typename T, bool R_CONTIG, bool VEC>
struct SlabLoader {
  static constexpr int BK = SimtCfg<T>::BK;
  static constexpr int W = VecT<T>::W;
  static constexpr int NV = kBM * BK / (kSimtThreads * W);  // vectors per thread (2)
  T reg[NV][W];

  __device__ __forceinline__ void load(const T* __restrict__ src, int64_t ld, int64_t r0, int64_t k0, int64_t R,
                                       int64_t K) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const int v = threadIdx.x + i * kSimtThreads;
      int r, k;
      if (R_CONTIG) {
        k = v / (kBM / W);
        r = (v % (kBM / W)) * W;
      } else {
        r = v / (BK / W);
        k = (v % (BK / W)) * W;
      }
      const int64_t gr = r0 + r, gk = k0 + k;
      if (R_CONTIG) {
        const T* p = src + gr + gk * ld;
        if (VEC && gk < K && gr + W <= R) {
          typename VecT<T>::V t = *reinterpret_cast<const typename VecT<T>::V*>(p);
          const T* tp = reinterpret_cast<const T*>(&t);
#pragma unroll
          for (int e = 0; e < W; ++e) reg[i][e] = tp[e];
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) reg[i][e] = (gk < K && gr + e < R) ? p[e] : T(0);
        }
      } else {
        const T* p = src + gk + gr * ld;
        if (VEC && gr < R && gk + W <= K) {
          typename VecT<T>::V t = *reinterpret_cast<const typename VecT<T>::V*>(p);
          const T* tp = reinterpret_cast<const T*>(&t);
#pragma unroll
          for (int e = 0; e < W; ++e) reg[i][e] = tp[e];
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) reg[i][e] = (gr < R && gk + e < K) ? p[e] : T(0);
        }
      }
    }
  }

  // smem slab is [BK][kBM] (k-major)
  __device__ __forceinline__ void store(T* s) const {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const int v = threadIdx.x + i * kSimtThreads;
      if (R_CONTIG) {
        const int k = v / (kBM / W), r = (v % (kBM / W)) * W;
        typename VecT<T>::V t;
        T* tp = reinterpret_cast<T*>(&t);
#pragma unroll
        for (int e = 0; e < W; ++e) tp[e] = reg[i][e];
        *reinterpret_cast<typename VecT<T>::V*>(s + k * kBM + r) = t;
      } else {
        const int r = v / (BK / W), k = (v % (BK / W)) * W;
#pragma unroll
        for (int e = 0; e < W; ++e) s[(k + e) * kBM + r] = reg[i][e];
      }
    }
  }
};

// TA / TB: operand stored transposed (k contiguous for A, n contiguous for B).
template <typename T, bool TA, bool TB, bool VA, bool VB, bool BETA0>
__global__ void __launch_bounds__(kSimtThreads) gemm_simt_kernel(GemmArgs<T> g) {
  constexpr int BK = SimtCfg<T>::BK;
  __shared__ __align__(16) T As[2][BK * kBM];
  __shared__ __align__(16) T Bs[2][BK * kBN];
  const int64_t bz = blockIdx.z;
  const T* A = g.a + bz * g.stride_a;
  const T* B = g.b + bz * g.stride_b;
  T* C = g.c + bz * g.stride_c;
  const int64_t m0 = int64_t(blockIdx.y) * kBM, n0 = int64_t(blockIdx.x) * kBN;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;

  // A slab rows run along M: contiguous when A is not transposed.
  SlabLoader<T, !TA, VA> la;
  // B slab rows run along N: contiguous when B is transposed.
  SlabLoader<T, TB, VB> lb;

  T acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = T(0);

  const int64_t K = g.k;
  const int64_t nk = (K + BK - 1) / BK;
  if (nk > 0) {
    la.load(A, g.lda, m0, 0, g.m, K);
    lb.load(B, g.ldb, n0, 0, g.n, K);
    la.store(As[0]);
    lb.store(Bs[0]);
    __syncthreads();
  }
  for (int64_t kt = 0; kt < nk; ++kt) {
    const int cur = kt & 1;
    if (kt + 1 < nk) {
      la.load(A, g.lda, m0, (kt + 1) * BK, g.m, K);
      lb.load(B, g.ldb, n0, (kt + 1) * BK, g.n, K);
    }
    const T* as = As[cur];
    const T* bs = Bs[cur];
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      T af[8], bf[8];
      constexpr int W = VecT<T>::W;
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int e = 0; e < 4; e += W) {
          typename VecT<T>::V va = *reinterpret_cast<const typename VecT<T>::V*>(as + k * kBM + q * 64 + ty * 4 + e);
          typename VecT<T>::V vb = *reinterpret_cast<const typename VecT<T>::V*>(bs + k * kBN + q * 64 + tx * 4 + e);
          const T* pa = reinterpret_cast<const T*>(&va);
          const T* pb = reinterpret_cast<const T*>(&vb);
#pragma unroll
          for (int w = 0; w < W; ++w) {
            af[q * 4 + e + w] = pa[w];
            bf[q * 4 + e + w] = pb[w];
          }
        }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fma(af[i], bf[j], acc[i][j]);
    }
    if (kt + 1 < nk) {
      la.store(As[cur ^ 1]);
      lb.store(Bs[cur ^ 1]);
    }
    __syncthreads();
  }

  // epilogue: C(i, j) = alpha*acc + beta*C, column-major
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int64_t gn = n0 + (j / 4) * 64 + tx * 4 + (j % 4);
    if (gn >= g.n) continue;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int64_t gm = m0 + (i / 4) * 64 + ty * 4 + (i % 4);
      if (gm >= g.m) continue;
      T* cp = C + gm + gn * g.ldc;
      T r = g.alpha * acc[i][j];
      if (!BETA0) r = fma(g.beta, *cp, r);
      *cp = r;
    }
  }
}

template <typename T, bool TA, bool TB, bool BETA0>
gbblas_status_t launch_simt_tb(gbblas_handle_t h, const GemmArgs<T>& g) {
  constexpr int W = VecT<T>::W;
  const bool va = (g.lda % W == 0) && aligned16(g.a) && (g.batch == 1 || g.stride_a % W == 0);
  const bool vb = (g.ldb % W == 0) && aligned16(g.b) && (g.batch == 1 || g.stride_b % W == 0);
  for (int64_t b0 = 0; b0 < g.batch; b0 += 65535) {
    GemmArgs<T> gg = g;
    gg.a = g.a + b0 * g.stride_a;
    gg.b = g.b + b0 * g.stride_b;
    gg.c = g.c + b0 * g.stride_c;
    const int64_t nb = g.batch - b0 < 65535 ? g.batch - b0 : 65535;
    dim3 grid(unsigned(cdiv(g.n, kBN)), unsigned(cdiv(g.m, kBM)), unsigned(nb));
    if (grid.y > 65535) return fail(GBBLAS_STATUS_UNSUPPORTED, "gemm: M too large for the SIMT grid");
    if (va && vb) gemm_simt_kernel<T, TA, TB, true, true, BETA0><<<grid, kSimtThreads, 0, h->stream>>>(gg);
    else if (va) gemm_simt_kernel<T, TA, TB, true, false, BETA0><<<grid, kSimtThreads, 0, h->stream>>>(gg);
    else if (vb) gemm_simt_kernel<T, TA, TB, false, true, BETA0><<<grid, kSimtThreads, 0, h->stream>>>(gg);
    else gemm_simt_kernel<T, TA, TB, false, false, BETA0><<<grid, kSimtThreads, 0, h->stream>>>(gg);
    GB_TRY(after_launch("gemm_simt"));
  }
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T>
gbblas_status_t launch_simt_any(gbblas_handle_t h, const GemmArgs<T>& g) {
  const bool b0 = g.beta == T(0);
#define GB_SIMT_CASE(TA, TB)                                              \
  if (g.ta == TA && g.tb == TB)                                           \
    return b0 ? launch_simt_tb<T, TA, TB, true>(h, g) : launch_simt_tb<T, TA, TB, false>(h, g);
  GB_SIMT_CASE(false, false)
  GB_SIMT_CASE(false, true)
  GB_SIMT_CASE(true, false)
  GB_SIMT_CASE(true, true)
#undef GB_SIMT_CASE
  return GBBLAS_STATUS_INVALID_ARG;
}

gbblas_status_t launch_gemm_simt(gbblas_handle_t h, const GemmArgs<float>& g) { return launch_simt_any(h, g); }
gbblas_status_t launch_gemm_simt(gbblas_handle_t h, const GemmArgs<double>& g) { return launch_simt_any(h, g); }

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

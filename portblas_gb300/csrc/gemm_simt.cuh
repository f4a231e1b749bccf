// gemm_simt.cuh — plain FP32 / FP64 GEMM on the CUDA cores (SIMT FMA).
//
// This is the "plain FP32" comparator of the split-BF16 tensor-core SGEMM and
// the FP64-pipe DGEMM.  It plays the role of portBLAS's Gemm<local, ...>
// kernel (src/operations/blas3/gemm_local.hpp:74-875), which stages A and B
// blocks in work-group local memory and accumulates a register tile with
// sycl::mad; the structure here is the usual CUDA one: a BM x BN CTA tile
// (128x128, 128x64, 64x128 or 64x64, 256 threads), k-major shared-memory
// slabs filled from registers (so any transpose is a register shuffle), a
// TM x TN register micro-tile per thread in 4x4 quadrants spaced BM/(TM/4)
// apart (conflict-free 128-bit shared loads), double buffering, and a fused
// alpha/beta epilogue alpha*acc + beta*C (gemm_ref.hpp:240-250); beta == 0
// never reads C (gemm_local.hpp:401-409).
//
// Batches run on gridDim.z; a split-K factor S adds S slices of K per
// problem on gridDim.z, each writing its partial tile to temp memory, and a
// fixed-order reduction kernel sums the slices and applies the epilogue
// (deterministic).
#pragma once
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

constexpr int kSimtThreads = 256;

// Loads one BK-deep slab of an operand tile of R rows into registers.
// Element (r, k) of the slab (r along M or N, k along K) lives at
// src[r + k*ld] when R_CONTIG (r contiguous) and at src[k + r*ld] otherwise.
template <typename T, int R, bool R_CONTIG, bool VEC>
struct SlabLoader {
  static constexpr int BK = SimtCfg<T>::BK;
  static constexpr int W = VecT<T>::W;
  static constexpr int NV = R * BK / (kSimtThreads * W);  // vectors per thread
  static_assert(NV >= 1 && NV * kSimtThreads * W == R * BK, "slab must split evenly over the CTA");
  T reg[NV][W];

  __device__ __forceinline__ void load(const T* __restrict__ src, int64_t ld, int64_t r0, int64_t k0, int64_t Rn,
                                       int64_t K) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const int v = threadIdx.x + i * kSimtThreads;
      int r, k;
      if (R_CONTIG) {
        k = v / (R / W);
        r = (v % (R / W)) * W;
      } else {
        r = v / (BK / W);
        k = (v % (BK / W)) * W;
      }
      const int64_t gr = r0 + r, gk = k0 + k;
      if (R_CONTIG) {
        const T* p = src + gr + gk * ld;
        if (VEC && gk < K && gr + W <= Rn) {
          typename VecT<T>::V t = *reinterpret_cast<const typename VecT<T>::V*>(p);
          const T* tp = reinterpret_cast<const T*>(&t);
#pragma unroll
          for (int e = 0; e < W; ++e) reg[i][e] = tp[e];
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) reg[i][e] = (gk < K && gr + e < Rn) ? p[e] : T(0);
        }
      } else {
        const T* p = src + gk + gr * ld;
        if (VEC && gr < Rn && gk + W <= K) {
          typename VecT<T>::V t = *reinterpret_cast<const typename VecT<T>::V*>(p);
          const T* tp = reinterpret_cast<const T*>(&t);
#pragma unroll
          for (int e = 0; e < W; ++e) reg[i][e] = tp[e];
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) reg[i][e] = (gr < Rn && gk + e < K) ? p[e] : T(0);
        }
      }
    }
  }

  // smem slab is [BK][R] (k-major)
  __device__ __forceinline__ void store(T* s) const {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const int v = threadIdx.x + i * kSimtThreads;
      if (R_CONTIG) {
        const int k = v / (R / W), r = (v % (R / W)) * W;
        typename VecT<T>::V t;
        T* tp = reinterpret_cast<T*>(&t);
#pragma unroll
        for (int e = 0; e < W; ++e) tp[e] = reg[i][e];
        *reinterpret_cast<typename VecT<T>::V*>(s + k * R + r) = t;
      } else {
        const int r = v / (BK / W), k = (v % (BK / W)) * W;
#pragma unroll
        for (int e = 0; e < W; ++e) s[(k + e) * R + r] = reg[i][e];
      }
    }
  }
};

// TA / TB: operand stored transposed (k contiguous for A, n contiguous for B).
// PARTIAL: split-K slice — writes the raw accumulator tile to `ws`
// ([batch][split][M][N], column-major M x N) instead of the epilogue.
template <typename T, int BM, int BN, int TM, int TN, bool TA, bool TB, bool VA, bool VB, bool PARTIAL>
__global__ void __launch_bounds__(kSimtThreads) gemm_simt_kernel(GemmArgs<T> g, int split, int64_t kchunk,
                                                                 T* __restrict__ ws) {
  constexpr int BK = SimtCfg<T>::BK;
  constexpr int NTX = BN / TN;
  static_assert((BM / TM) * (BN / TN) == kSimtThreads, "micro-tile layout must cover 256 threads");
  __shared__ __align__(16) T As[2][BK * BM];
  __shared__ __align__(16) T Bs[2][BK * BN];
  const int64_t bz = blockIdx.z / split;
  const int ks = blockIdx.z % split;
  const T* A = g.a + bz * g.stride_a;
  const T* B = g.b + bz * g.stride_b;
  const int64_t m0 = int64_t(blockIdx.y) * BM, n0 = int64_t(blockIdx.x) * BN;
  const int tx = threadIdx.x % NTX, ty = threadIdx.x / NTX;
  const int64_t kbeg = int64_t(ks) * kchunk;
  const int64_t kend = min(g.k, kbeg + kchunk);

  // A slab rows run along M: contiguous when A is not transposed.
  SlabLoader<T, BM, !TA, VA> la;
  // B slab rows run along N: contiguous when B is transposed.
  SlabLoader<T, BN, TB, VB> lb;

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

  const int64_t nk = kend > kbeg ? (kend - kbeg + BK - 1) / BK : 0;
  if (nk > 0) {
    la.load(A, g.lda, m0, kbeg, g.m, kend);
    lb.load(B, g.ldb, n0, kbeg, g.n, kend);
    la.store(As[0]);
    lb.store(Bs[0]);
    __syncthreads();
  }
  constexpr int W = VecT<T>::W;
  constexpr int QM = TM / 4, QN = TN / 4;  // 4x4 quadrants per thread
  for (int64_t kt = 0; kt < nk; ++kt) {
    const int cur = kt & 1;
    if (kt + 1 < nk) {
      la.load(A, g.lda, m0, kbeg + (kt + 1) * BK, g.m, kend);
      lb.load(B, g.ldb, n0, kbeg + (kt + 1) * BK, g.n, kend);
    }
    const T* as = As[cur];
    const T* bs = Bs[cur];
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      T af[TM], bf[TN];
#pragma unroll
      for (int q = 0; q < QM; ++q)
#pragma unroll
        for (int e = 0; e < 4; e += W) {
          typename VecT<T>::V va =
              *reinterpret_cast<const typename VecT<T>::V*>(as + k * BM + q * (BM / QM) + ty * 4 + e);
          const T* pa = reinterpret_cast<const T*>(&va);
#pragma unroll
          for (int w = 0; w < W; ++w) af[q * 4 + e + w] = pa[w];
        }
#pragma unroll
      for (int q = 0; q < QN; ++q)
#pragma unroll
        for (int e = 0; e < 4; e += W) {
          typename VecT<T>::V vb =
              *reinterpret_cast<const typename VecT<T>::V*>(bs + k * BN + q * (BN / QN) + tx * 4 + e);
          const T* pb = reinterpret_cast<const T*>(&vb);
#pragma unroll
          for (int w = 0; w < W; ++w) bf[q * 4 + e + w] = pb[w];
        }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(af[i], bf[j], acc[i][j]);
    }
    if (kt + 1 < nk) {
      la.store(As[cur ^ 1]);
      lb.store(Bs[cur ^ 1]);
    }
    __syncthreads();
  }

  if (PARTIAL) {
    T* W0 = ws + (bz * split + ks) * g.m * g.n;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t gn = n0 + (j / 4) * (BN / QN) + tx * 4 + (j % 4);
      if (gn >= g.n) continue;
#pragma unroll
      for (int i = 0; i < TM; ++i) {
        const int64_t gm = m0 + (i / 4) * (BM / QM) + ty * 4 + (i % 4);
        if (gm < g.m) W0[gm + gn * g.m] = acc[i][j];
      }
    }
    return;
  }
  // C is read one column of the micro-tile at a time, all TM loads before
  // the stores, so the loads overlap (a store may alias a later load when
  // ldc == 0, so the compiler cannot reorder them itself)
  T* C = g.c + bz * g.stride_c;
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    const int64_t gn = n0 + (j / 4) * (BN / QN) + tx * 4 + (j % 4);
    if (gn >= g.n) continue;
    T cv[TM];
    if (g.beta != T(0)) {
#pragma unroll
      for (int i = 0; i < TM; ++i) {
        const int64_t gm = m0 + (i / 4) * (BM / QM) + ty * 4 + (i % 4);
        cv[i] = gm < g.m ? C[gm + gn * g.ldc] : T(0);
      }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int64_t gm = m0 + (i / 4) * (BM / QM) + ty * 4 + (i % 4);
      if (gm >= g.m) continue;
      T r = g.alpha * acc[i][j];
      if (g.beta != T(0)) r = fma(g.beta, cv[i], r);
      C[gm + gn * g.ldc] = r;
    }
  }
}

// Sums the split-K slices in slice order and applies alpha/beta.
template <typename T>
__global__ void splitk_reduce_kernel(GemmArgs<T> g, int split, const T* __restrict__ ws, int64_t nb) {
  const int64_t mn = g.m * g.n;
  const int64_t total = mn * nb;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t b = e / mn, r = e % mn;
    const int64_t gm = r % g.m, gn = r / g.m;
    const T* p = ws + b * split * mn + r;
    T s = p[0];
    for (int q = 1; q < split; ++q) s += p[q * mn];
    T* cp = g.c + b * g.stride_c + gm + gn * g.ldc;
    T v = g.alpha * s;
    if (g.beta != T(0)) v = fma(g.beta, *cp, v);
    *cp = v;
  }
}

template <typename T, int BM, int BN, int TM, int TN, bool TA, bool TB>
gbblas_status_t launch_simt_tile(gbblas_handle_t h, const GemmArgs<T>& g, int split) {
  constexpr int W = VecT<T>::W;
  constexpr int BK = SimtCfg<T>::BK;
  const bool va = (g.lda % W == 0) && aligned16(g.a) && (g.batch == 1 || g.stride_a % W == 0);
  const bool vb = (g.ldb % W == 0) && aligned16(g.b) && (g.batch == 1 || g.stride_b % W == 0);
  if (split < 1 || g.k <= BK) split = 1;
  const int64_t kchunk = split > 1 ? cdiv(cdiv(g.k, split), BK) * BK : g.k;
  if (split > 1) split = int(cdiv(g.k, kchunk));  // drop empty slices
  T* ws = nullptr;
  // batch slab so grid.z stays within 65535 and the workspace bounded
  int64_t bmax = 65535 / split;
  if (split > 1) {
    const int64_t per = int64_t(split) * g.m * g.n;
    const int64_t cap = (int64_t(1) << 28) / (per > 0 ? per : 1);  // <= 1 GiB of FP32 partials
    if (cap < 1) return fail(GBBLAS_STATUS_UNSUPPORTED, "gemm: split-K workspace too large");
    if (bmax > cap) bmax = cap;
    void* tmp;
    GB_TRY(temp_acquire(h, sizeof(T) * size_t(per) * size_t(g.batch < bmax ? g.batch : bmax), &tmp));
    ws = static_cast<T*>(tmp);
  }
  for (int64_t b0 = 0; b0 < g.batch; b0 += bmax) {
    GemmArgs<T> gg = g;
    gg.a = g.a + b0 * g.stride_a;
    gg.b = g.b + b0 * g.stride_b;
    gg.c = g.c + b0 * g.stride_c;
    const int64_t nb = g.batch - b0 < bmax ? g.batch - b0 : bmax;
    dim3 grid(unsigned(cdiv(g.n, BN)), unsigned(cdiv(g.m, BM)), unsigned(nb * split));
    if (grid.y > 65535) return fail(GBBLAS_STATUS_UNSUPPORTED, "gemm: M too large for the SIMT grid");
#define GB_SIMT_LAUNCH(VA_, VB_)                                                                     \
  if (split > 1)                                                                                     \
    gemm_simt_kernel<T, BM, BN, TM, TN, TA, TB, VA_, VB_, true>                                      \
        <<<grid, kSimtThreads, 0, h->stream>>>(gg, split, kchunk, ws);                              \
  else                                                                                               \
    gemm_simt_kernel<T, BM, BN, TM, TN, TA, TB, VA_, VB_, false>                                     \
        <<<grid, kSimtThreads, 0, h->stream>>>(gg, split, kchunk, ws);
    if (va && vb) { GB_SIMT_LAUNCH(true, true) }
    else if (va) { GB_SIMT_LAUNCH(true, false) }
    else if (vb) { GB_SIMT_LAUNCH(false, true) }
    else { GB_SIMT_LAUNCH(false, false) }
#undef GB_SIMT_LAUNCH
    GB_TRY(after_launch("gemm_simt"));
    if (split > 1) {
      const int64_t total = g.m * g.n * nb;
      const int64_t blocks = cdiv(total, 256) < int64_t(h->sm_count) * 8 ? cdiv(total, 256) : int64_t(h->sm_count) * 8;
      splitk_reduce_kernel<T><<<unsigned(blocks), 256, 0, h->stream>>>(gg, split, ws, nb);
      GB_TRY(after_launch("splitk_reduce"));
    }
  }
  return GBBLAS_STATUS_SUCCESS;
}

template <typename T, int BM, int BN, int TM, int TN>
gbblas_status_t launch_simt_cfg(gbblas_handle_t h, const GemmArgs<T>& g, int split) {
#define GB_SIMT_CASE(TA, TB) \
  if (g.ta == TA && g.tb == TB) return launch_simt_tile<T, BM, BN, TM, TN, TA, TB>(h, g, split);
  GB_SIMT_CASE(false, false)
  GB_SIMT_CASE(false, true)
  GB_SIMT_CASE(true, false)
  GB_SIMT_CASE(true, true)
#undef GB_SIMT_CASE
  return GBBLAS_STATUS_INVALID_ARG;
}

}  // namespace gb

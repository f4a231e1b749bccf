// grouped_tc.cuh — tensor-core (tcgen05) tile kernel of the grouped GEMM.
//
// Same scheduler as the SIMT grouped kernel (persistent CTAs, global atomic
// tile counter, binary search over per-problem tile prefix sums), but each
// 128 x 64 output tile runs on tcgen05.mma with a TMEM accumulator.  Grouped
// problems have per-problem pointers, leading dimensions and transposes, so
// operand tiles cannot come from one tensor map: the 128 threads of the CTA
// gather them with ordinary loads (coalesced along whichever dimension is
// contiguous), convert them to BF16 terms (FP32 inputs are split into three
// terms, exact residuals, as in gemm_tc.cu) and store them in the same
// 128-byte-swizzled K-major layout TMA would produce, so the MMA descriptors
// are those of the TMA-fed kernel.  A proxy fence publishes the generic-proxy
// stores to the tensor core before the stage's mbarrier arrival.
//
// Per k-block (64) and stage: P A-term tiles (128 x 64) and P B-term tiles
// (64 x 64); two stages; 256 threads gather.  Thread 0 issues the MMAs (all
// term pairs with a + b <= P - 1) and commits each stage back to the loaders.
// Every 8 k-blocks the TMEM accumulator is promoted into FP32 registers (warp
// w holds rows 32*(w%4).. and 32 of the 64 columns) so long K keeps
// FP32-level accuracy.
#pragma once

#include <cuda_bf16.h>

#include "tc_ptx.cuh"

namespace gb {

constexpr int kGtBM = 128, kGtBN = 64, kGtBK = 64, kGtThreads = 256, kGtChunk = 8;

template <int P>
struct GtCfg {
  static constexpr int A_TILE = kGtBM * kGtBK * 2;  // 16 KB
  static constexpr int B_TILE = kGtBN * kGtBK * 2;  //  8 KB
  static constexpr int STAGE = P * (A_TILE + B_TILE);
  static constexpr int STAGES = 2;
  static constexpr int SMEM = STAGES * STAGE + 1024 + 128;
  static constexpr int NPAIRS = P == 1 ? 1 : (P == 2 ? 3 : 6);
};

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// byte offset of 16-byte chunk c (k / 8) of row r in a 128 B-swizzled,
// K-major tile (8-row groups 1024 B apart, chunk index XOR row % 8)
__device__ __forceinline__ uint32_t sw128_offset(int r, int c) {
  return uint32_t((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

template <typename T>
__device__ __forceinline__ float ld_f32(const T* p);
template <>
__device__ __forceinline__ float ld_f32<float>(const float* p) { return __ldg(p); }
template <>
__device__ __forceinline__ float ld_f32<__nv_bfloat16>(const __nv_bfloat16* p) { return __bfloat162float(*p); }

__device__ __forceinline__ void load_vec8(const float* p, float* v) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p)), b = __ldg(reinterpret_cast<const float4*>(p) + 1);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
__device__ __forceinline__ void load_vec8(const __nv_bfloat16* p, float* v) {
  const uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
  const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&a);
#pragma unroll
  for (int e = 0; e < 8; ++e) v[e] = __bfloat162float(h[e]);
}

// Gathers NCH chunks of 8 consecutive k of one row (global row gr) of an
// operand whose element (row, k) is at src[row*srow + k*sk]: load() issues
// every global load of the k-block first (so they are all in flight
// together), store() splits the values into P BF16 terms and writes one
// 16-byte swizzled chunk per term.
template <typename T, int NCH>
struct RowGather {
  float v[NCH][8];
  __device__ __forceinline__ void load(const T* src, int64_t srow, int64_t sk, int64_t gr, int64_t rows, int64_t k0,
                                       int64_t K, int c0) {
    const bool row_ok = gr < rows;
    const T* p = src + (row_ok ? gr : 0) * srow + (k0 + int64_t(c0) * 8) * sk;
    const int64_t kleft = K - (k0 + int64_t(c0) * 8);  // valid k from the first chunk on
    if (row_ok && kleft >= NCH * 8) {
      if (sk == 1 && (reinterpret_cast<uintptr_t>(p) & 15) == 0) {
        // K contiguous and 16-byte aligned: 128-bit loads
#pragma unroll
        for (int c = 0; c < NCH; ++c) load_vec8(p + c * 8, v[c]);
      } else {
        // interior: no per-element bounds checks, 32-bit strides
        const int s = int(sk);
#pragma unroll
        for (int c = 0; c < NCH; ++c)
#pragma unroll
          for (int e = 0; e < 8; ++e) v[c][e] = ld_f32<T>(p + (c * 8 + e) * s);
      }
      return;
    }
#pragma unroll
    for (int c = 0; c < NCH; ++c)
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int64_t kk = int64_t(c) * 8 + e;
        v[c][e] = (row_ok && kk < kleft) ? ld_f32<T>(p + kk * sk) : 0.f;
      }
  }
  template <int P>
  __device__ __forceinline__ void store(uint8_t* tile0, int tile_bytes, int r, int c0) {
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
      const uint32_t off = sw128_offset(r, c0 + c);
#pragma unroll
      for (int p = 0; p < P; ++p) {
        __align__(16) __nv_bfloat16 h[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          h[e] = __float2bfloat16_rn(v[c][e]);
          v[c][e] -= __bfloat162float(h[e]);  // exact residual for the next term
        }
        *reinterpret_cast<uint4*>(tile0 + p * tile_bytes + off) = *reinterpret_cast<const uint4*>(h);
      }
    }
  }
};

enum : int { kErrGtFull = 401, kErrGtEmpty = 402, kErrGtAcc = 403 };

// probs / count / total_tiles / counters: as grouped_gemm_kernel (grouped.cu),
// with tiles of 128 x 64.
template <typename T, int P, class Prob>
__global__ void __launch_bounds__(kGtThreads, 2)
    grouped_tc_kernel(const Prob* __restrict__ probs, int count, int64_t total_tiles,
                      unsigned long long* __restrict__ counters, int* __restrict__ err) {
  using Cfg = GtCfg<P>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Cfg::STAGES * Cfg::STAGE);
  uint64_t* empty = full + Cfg::STAGES;
  uint64_t* accb = empty + Cfg::STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accb + 1);
  __shared__ long long tile_sh;
  __shared__ int prob_sh;
  __shared__ int abort_sh;

  const int t = threadIdx.x, warp = t >> 5;
  if (t == 0) {
    for (int s = 0; s < Cfg::STAGES; ++s) {
      tc::mbar_init(&full[s], kGtThreads);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(accb, 1);
    tc::fence_mbar_init();
    abort_sh = 0;
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, kGtBN);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  constexpr uint32_t idesc = tc::idesc_bf16_f32(kGtBM, kGtBN);

  uint32_t it = 0;    // stage iterations so far (all threads agree)
  uint32_t nacc = 0;  // accumulator commits so far
  for (;;) {
    if (t == 0) {
      tile_sh = (long long)atomicAdd(&counters[0], 1ull);
      if (tile_sh < total_tiles) {
        int lo = 0, hi = count - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (probs[mid].tile_start <= tile_sh) lo = mid; else hi = mid - 1;
        }
        prob_sh = lo;
      }
    }
    __syncthreads();
    const long long tile = tile_sh;
    if (tile >= total_tiles || abort_sh) break;
    const Prob& pr = probs[prob_sh];
    const int local = int(tile - pr.tile_start);
    const int64_t m0 = int64_t(local / pr.tiles_n) * kGtBM, n0 = int64_t(local % pr.tiles_n) * kGtBN;
    const T* A = static_cast<const T*>(pr.a);
    const T* B = static_cast<const T*>(pr.b);
    // A(m, k) = ta ? A[k + m*lda] : A[m + k*lda];  B as rows n: (tb ? B[n + k*ldb] : B[k + n*ldb])
    const int64_t a_srow = pr.ta ? pr.lda : 1, a_sk = pr.ta ? 1 : pr.lda;
    const int64_t b_srow = pr.tb ? 1 : pr.ldb, b_sk = pr.tb ? pr.ldb : 1;
    const int nk = int((pr.k + kGtBK - 1) / kGtBK);
    // warp w: TMEM lanes 32*(w%4) (rows), columns 32*(w/4) .. +31 of the tile
    const int half = warp >> 2;
    float sum[kGtBN / 2];
#pragma unroll
    for (int i = 0; i < kGtBN / 2; ++i) sum[i] = 0.f;
    RowGather<T, 4> ga;
    RowGather<T, 2> gbt;
    bool ok = true;
    for (int kb = 0; kb < nk && ok; ++kb, ++it) {
      const int s = it % Cfg::STAGES;
      const uint32_t ph = (it / Cfg::STAGES) & 1;
      uint8_t* st = smem + s * Cfg::STAGE;
      const int64_t k0 = int64_t(kb) * kGtBK;
      // A: 128 rows x 8 chunks, thread t takes row t%128, chunks 4*(t/128)..+3;
      // B: 64 rows x 8 chunks, thread t takes row t%64, chunks 2*(t/64)..+1.
      // The loads go out before the wait for the stage, overlapping the MMAs
      // still reading it.
      ga.load(A, a_srow, a_sk, m0 + (t & 127), pr.m, k0, pr.k, (t >> 7) * 4);
      gbt.load(B, b_srow, b_sk, n0 + (t & 63), pr.n, k0, pr.k, (t >> 6) * 2);
      if (!tc::mbar_wait(&empty[s], ph ^ 1)) {
        if (t == 0) atomicExch(err, kErrGtEmpty);
        ok = false;
        break;
      }
      ga.template store<P>(st, Cfg::A_TILE, t & 127, (t >> 7) * 4);
      gbt.template store<P>(st + P * Cfg::A_TILE, Cfg::B_TILE, t & 63, (t >> 6) * 2);
      fence_proxy_async_smem();
      tc::mbar_arrive(&full[s]);
      const bool chunk_end = (kb + 1 == nk) || ((kb + 1) % kGtChunk == 0);
      if (t == 0) {
        if (!tc::mbar_wait(&full[s], ph)) {
          atomicExch(err, kErrGtFull);
          abort_sh = 1;
        } else {
          tc::tc_fence_after();
#pragma unroll
          for (int q = 0; q < Cfg::NPAIRS; ++q) {
            const int pa = (q == 2 || q == 4) ? 1 : (q == 5 ? 2 : 0);
            const int pb = (q == 1 || q == 4) ? 1 : (q == 3 ? 2 : 0);
            const uint64_t ad = tc::sdesc_kmajor_sw128(tc::smem_u32(st + pa * Cfg::A_TILE));
            const uint64_t bd = tc::sdesc_kmajor_sw128(tc::smem_u32(st + P * Cfg::A_TILE + pb * Cfg::B_TILE));
#pragma unroll
            for (int j = 0; j < kGtBK / 16; ++j)
              tc::mma_bf16(tmem, ad + 2 * j, bd + 2 * j, idesc, (kb % kGtChunk) != 0 || q != 0 || j != 0);
          }
          tc::mma_commit(&empty[s]);
          if (chunk_end) tc::mma_commit(accb);
        }
      }
      if (chunk_end) {
        // promote the chunk accumulator into registers
        if (!tc::mbar_wait(accb, nacc & 1)) {
          if (t == 0) atomicExch(err, kErrGtAcc);
          ok = false;
        }
        ++nacc;
        tc::tc_fence_after();
        if (ok) {
          uint32_t r[32];
          tc::tmem_ld_32x32b_x32(tmem + (uint32_t((warp & 3) * 32) << 16) + uint32_t(half * 32), r);
          tc::tmem_ld_wait();
#pragma unroll
          for (int i = 0; i < 32; ++i) sum[i] += __uint_as_float(r[i]);
        }
        tc::tc_fence_before();
        __syncthreads();  // everyone has read TMEM before the next chunk's MMAs
        if (abort_sh) ok = false;
      }
    }
    if (!ok) {
      if (t == 0) abort_sh = 1;
      __syncthreads();
      break;
    }
    // epilogue: row m0 + 32*(warp%4) + lane, columns n0 + 32*half + i
    const int64_t gm = m0 + (warp & 3) * 32 + (t & 31);
    if (gm < pr.m) {
#pragma unroll
      for (int i = 0; i < kGtBN / 2; ++i) {
        const int64_t gn = n0 + half * 32 + i;
        if (gn < pr.n) {
          float* cp = pr.c + gm + gn * pr.ldc;
          float v = pr.alpha * sum[i];
          if (pr.beta != 0.f) v = fmaf(pr.beta, *cp, v);
          *cp = v;
        }
      }
    }
    __syncthreads();
  }
  // let the last MMAs and copies settle, free TMEM, reset the scheduler
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, kGtBN);
  }
  if (t == 0) {
    __threadfence();
    const unsigned long long done = atomicAdd(&counters[1], 1ull);
    if (done == gridDim.x - 1) {
      counters[0] = 0ull;
      counters[1] = 0ull;
      __threadfence();
    }
  }
}

}  // namespace gb

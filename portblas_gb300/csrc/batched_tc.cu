// batched_tc.cu — strided batches of small FP32 problems (M, N, K <= 64) on
// the tcgen05 tensor cores.
//
// Two problems p, q share one M128 x N128 tile: A rows 0..63 are A_p and
// 64..127 A_q, B rows (the N dimension) 0..63 are B_p and 64..127 B_q, so
// the diagonal 64 x 64 blocks of D are A_p B_p and A_q B_q (the off-diagonal
// blocks are computed and dropped: the tensor pipe has room to spare, this
// path is bound by HBM).  A pair is processed in two steps of 32 k each, so
// the rings hold several steps:
//   warp 0      TMA producer: per step the raw FP32 k-halves of A_p, A_q,
//               B_p, B_q (8 KB each: one 32 x 64 box when the operand runs
//               along k, else two 32 x 32 boxes; 128-byte swizzle;
//               zero-filled outside M, N, K and past the end of the batch)
//               into a four-stage ring;
//   warps 2-9   converters: the three BF16 terms of every element (exact
//               residuals) into one of two term stages, K-major with the
//               64-byte swizzle, reading the raw tile along k or, for
//               operands whose rows run along M / N, transposing it; a proxy
//               fence and one arrival per warp publish the stage;
//   warp 1      allocates TMEM and issues the six term products as four
//               MMAs per 16 k (a0 x [b0; b1] and a1 x [b0; b1] as N = 256,
//               a0 b2 and a2 b0 into the second column half), both steps of a
//               pair into one of two accumulators, so the next pair runs
//               while the epilogue drains this one;
//   warps 10-17 epilogue: two warps per TMEM lane quarter, each thread one
//               row of one problem (TMEM lane r < 64: problem p, columns
//               0..63; else q, columns 64..127) and 32 of its 64 columns,
//               both column halves summed, alpha / beta, stores to C.  (With
//               four warps the epilogue was busy 77% of the kernel and held
//               the accumulators, the term stages and the raw ring behind
//               it; per-role clock counters.)
// Every mbarrier wait is bounded; a wait that gives up records an error
// code, the producer waits for its copies in flight and TMEM is freed.
#include <cuda_bf16.h>

#include "common.cuh"
#include "gemm_internal.cuh"
#include "tc_ptx.cuh"

namespace gb {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn tensor_map_encoder();  // gemm_tc.cu

constexpr int kBtConvWarps = 8, kBtEpiWarps = 8, kBtFirstConv = 2, kBtFirstEpi = kBtFirstConv + kBtConvWarps;
constexpr int kBtThreads = (kBtFirstEpi + kBtEpiWarps) * 32;
constexpr int kBtRawSlot = 64 * 32 * 4;        // one operand's raw FP32 k-half (8 KB)
constexpr int kBtRawStage = 4 * kBtRawSlot;    // A_p, A_q, B_p, B_q
constexpr int kBtRawStages = 4;
constexpr int kBtTermTile = 128 * 32 * 2;      // one BF16 term of the stacked A (or B): 128 rows x 32 k
constexpr int kBtTermStage = 6 * kBtTermTile;  // 3 terms of A, then 3 of B
constexpr int kBtTermStages = 2;
constexpr int kBtAcc = 256;                    // TMEM columns of one accumulator (two column halves)
constexpr int kBtSmem = kBtRawStages * kBtRawStage + kBtTermStages * kBtTermStage + 1024 + 256;
static_assert(kBtSmem <= 227 * 1024, "shared memory budget");

enum : int { kErrBtProducer = 501, kErrBtConv = 502, kErrBtMma = 503, kErrBtEpi = 504, kErrBtDrain = 505 };

struct BtArgs {
  int M, N, K;
  int64_t batch, pairs;
  float alpha, beta;
  float* c;
  int64_t ldc, stride_c;
};

// One 8-element k group (g = 0..3 of the step's 32 k) of row r (0..63) of a
// raw operand k-half, as floats.  kcontig: the tile's rows are r, k
// contiguous (one 64 x 32 box); else its rows are k, r contiguous (two
// 32 x 32 boxes, by r).  As TMA wrote them with the 128-byte swizzle
// (16-byte chunk c of row x at c ^ (x % 8)).
__device__ __forceinline__ void bt_read8(const uint8_t* slot, bool kcontig, int r, int g, float (&x)[8]) {
  if (kcontig) {
    const uint8_t* row = slot + r * 128;
    const int c0 = 2 * g;
    const float4 v0 = *reinterpret_cast<const float4*>(row + ((c0 ^ (r & 7)) << 4));
    const float4 v1 = *reinterpret_cast<const float4*>(row + (((c0 + 1) ^ (r & 7)) << 4));
    x[0] = v0.x; x[1] = v0.y; x[2] = v0.z; x[3] = v0.w;
    x[4] = v1.x; x[5] = v1.y; x[6] = v1.z; x[7] = v1.w;
  } else {
    const uint8_t* box = slot + (r >> 5) * 4096;
    const int col = r & 31;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int k = 8 * g + e;
      x[e] = *reinterpret_cast<const float*>(box + k * 128 + (((col >> 2) ^ (k & 7)) << 4) + (col & 3) * 4);
    }
  }
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(kBtThreads, 1)
    batched_tc_kernel(const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_b,
                      BtArgs g, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* raw = smem;                                   // [4][A_p, A_q, B_p, B_q] k-halves
  uint8_t* terms = smem + kBtRawStages * kBtRawStage;    // [2][a0 a1 a2 b0 b1 b2]
  uint64_t* rfull = reinterpret_cast<uint64_t*>(terms + kBtTermStages * kBtTermStage);
  uint64_t* rempty = rfull + kBtRawStages;
  uint64_t* tfull = rempty + kBtRawStages;    // [2] term stage written
  uint64_t* tempty = tfull + kBtTermStages;   // [2] term stage read by the MMAs
  uint64_t* afull = tempty + kBtTermStages;   // [2] accumulator ready
  uint64_t* aempty = afull + 2;               // [2] accumulator drained
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(aempty + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kBtRawStages; ++s) {
      tc::mbar_init(&rfull[s], 1);
      tc::mbar_init(&rempty[s], kBtConvWarps);
    }
    for (int s = 0; s < kBtTermStages; ++s) {
      tc::mbar_init(&tfull[s], kBtConvWarps);
      tc::mbar_init(&tempty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&afull[b], 1);
      tc::mbar_init(&aempty[b], kBtEpiWarps);  // one arrival per epilogue warp
    }
    tc::fence_mbar_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tmem_slot, 2 * kBtAcc);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const int64_t npairs = g.pairs;

  if (warp == 0) {
    // ------------------------------------------------------------ producer --
    if (lane == 0) {
      tc::tma_prefetch_desc(&tma_a);
      tc::tma_prefetch_desc(&tma_b);
      uint32_t it = 0;  // steps issued
      bool ok = true;
      for (int64_t pr = blockIdx.x; pr < npairs && ok; pr += gridDim.x) {
        for (int kh = 0; kh < 2; ++kh, ++it) {
          const int s = it % kBtRawStages;
          if (!tc::mbar_wait(&rempty[s], ((it / kBtRawStages) & 1) ^ 1)) {
            atomicExch(err, kErrBtProducer);
            ok = false;
            break;
          }
          tc::mbar_arrive_expect_tx(&rfull[s], kBtRawStage);
          uint8_t* st = raw + s * kBtRawStage;
#pragma unroll
          for (int slot = 0; slot < 4; ++slot) {
            const int prob = int(2 * pr + (slot & 1));  // past the batch: the box is zero-filled
            const bool isA = slot < 2;
            const CUtensorMap* map = isA ? &tma_a : &tma_b;
            const bool kcontig = isA ? TA : !TB;
            uint8_t* d = st + slot * kBtRawSlot;
            if (kcontig) {
              tc::tma_load_3d(d, map, &rfull[s], 32 * kh, 0, prob);  // 32 k x 64 rows
            } else {
              tc::tma_load_3d(d, map, &rfull[s], 0, 32 * kh, prob);  // 32 rows x 32 k, twice
              tc::tma_load_3d(d + 4096, map, &rfull[s], 32, 32 * kh, prob);
            }
          }
        }
      }
      // drain: every copy this thread issued has landed before the CTA exits
      for (uint32_t j = it > uint32_t(kBtRawStages) ? it - kBtRawStages : 0u; j < it; ++j)
        if (!tc::mbar_wait(&rfull[j % kBtRawStages], (j / kBtRawStages) & 1)) {
          atomicExch(err, kErrBtDrain);
          break;
        }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer --
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 128);
      constexpr uint32_t idesc2 = tc::idesc_bf16_f32(128, 256);
      uint32_t it = 0, np = 0;  // steps, pairs
      bool ok = true;
      for (int64_t pr = blockIdx.x; pr < npairs && ok; pr += gridDim.x, ++np) {
        const int b = np & 1;
        if (!tc::mbar_wait(&aempty[b], ((np >> 1) & 1) ^ 1)) {
          atomicExch(err, kErrBtMma);
          break;
        }
        const uint32_t acc = tmem + uint32_t(b * kBtAcc), acc2 = acc + 128u;
        for (int kh = 0; kh < 2; ++kh, ++it) {
          const int s = it % kBtTermStages;
          if (!tc::mbar_wait(&tfull[s], (it / kBtTermStages) & 1)) {
            atomicExch(err, kErrBtMma);
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t st = tc::smem_u32(terms + s * kBtTermStage);
          const uint64_t a0 = tc::sdesc_kmajor_sw64(st), a1 = tc::sdesc_kmajor_sw64(st + kBtTermTile);
          const uint64_t a2 = tc::sdesc_kmajor_sw64(st + 2 * kBtTermTile);
          const uint64_t b01 = tc::sdesc_kmajor_sw64(st + 3 * kBtTermTile);
          const uint64_t b2 = tc::sdesc_kmajor_sw64(st + 5 * kBtTermTile);
#pragma unroll
          for (int j = 0; j < 2; ++j) {  // K = 16 per MMA: +32 bytes in the swizzled row
            tc::mma_bf16(acc, a0 + 2 * j, b01 + 2 * j, idesc2, kh != 0 || j != 0);
            tc::mma_bf16(acc, a1 + 2 * j, b01 + 2 * j, idesc2, true);
            tc::mma_bf16(acc2, a0 + 2 * j, b2 + 2 * j, idesc, true);
            tc::mma_bf16(acc2, a2 + 2 * j, b01 + 2 * j, idesc, true);
          }
          tc::mma_commit(&tempty[s]);
        }
        if (ok) tc::mma_commit(&afull[b]);
      }
    }
  } else if (warp < kBtFirstEpi) {
    // ---------------------------------------------------------- converters --
    const int ct = threadIdx.x - 32 * kBtFirstConv;  // 0..255
    uint32_t it = 0;
    bool ok = true;
    for (int64_t pr = blockIdx.x; pr < npairs && ok; pr += gridDim.x) {
      for (int kh = 0; kh < 2; ++kh, ++it) {
        const int s = it % kBtRawStages, ts = it % kBtTermStages;
        uint32_t got = 1;
        if (lane == 0)
          got = tc::mbar_wait(&rfull[s], (it / kBtRawStages) & 1) &&
                tc::mbar_wait(&tempty[ts], ((it / kBtTermStages) & 1) ^ 1);
        got = __shfl_sync(0xffffffffu, got, 0);
        __syncwarp();
        if (!got) {
          if (lane == 0) atomicExch(err, kErrBtConv);
          ok = false;
          break;
        }
        const uint8_t* st = raw + s * kBtRawStage;
        uint8_t* tt = terms + ts * kBtTermStage;
#pragma unroll
        for (int slot = 0; slot < 4; ++slot) {
          const bool isA = slot < 2;
          const bool kcontig = isA ? TA : !TB;  // A 't' and B 'n' run along k
          const int task = ct;                  // 256 (row, k group) tasks per operand k-half
          const int r = task & 63, grp = task >> 6;
          float x[8];
          bt_read8(st + slot * kBtRawSlot, kcontig, r, grp, x);
          uint32_t w[3][4];
#pragma unroll
          for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const __nv_bfloat162 h2 = __floats2bfloat162_rn(x[2 * e], x[2 * e + 1]);
              w[p][e] = *reinterpret_cast<const uint32_t*>(&h2);
              if (p < 2) {
                x[2 * e] -= __uint_as_float(w[p][e] << 16);
                x[2 * e + 1] -= __uint_as_float(w[p][e] & 0xffff0000u);
              }
            }
          // K-major term rows of 32 k (64 bytes), 64-byte swizzle
          const int R = (slot & 1) * 64 + r;
          const uint32_t off = uint32_t(R) * 64u + (uint32_t(grp ^ ((R >> 1) & 3)) << 4);
          uint8_t* d = tt + (isA ? 0 : 3 * kBtTermTile) + off;
#pragma unroll
          for (int p = 0; p < 3; ++p)
            *reinterpret_cast<uint4*>(d + p * kBtTermTile) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
        }
        tc::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) {
          tc::mbar_arrive(&tfull[ts]);
          tc::mbar_arrive(&rempty[s]);
        }
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue --
    const int q = warp & 3;  // TMEM lanes 32q .. 32q+31
    const int c0 = 32 * ((warp - kBtFirstEpi) >> 2);  // this warp's 32 of the 64 columns
    const int R = 32 * q + lane;
    const int i = R & 63, half = R >> 6;  // row of problem 2*pair + half
    uint32_t it = 0;
    for (int64_t pr = blockIdx.x; pr < npairs; pr += gridDim.x, ++it) {
      const int b = it & 1;
      if (!tc::mbar_wait(&afull[b], (it >> 1) & 1)) {
        if (lane == 0) atomicExch(err, kErrBtEpi);
        break;
      }
      tc::tc_fence_after();
      float sum[32];
      {
        uint32_t v[32], u[32];
        const uint32_t base = tmem + (uint32_t(32 * q) << 16) + uint32_t(b * kBtAcc + half * 64 + c0);
        tc::tmem_ld_32x32b_x32(base, v);
        tc::tmem_ld_32x32b_x32(base + 128u, u);  // second column half: the cross terms
        tc::tmem_ld_wait();
#pragma unroll
        for (int j = 0; j < 32; ++j) sum[j] = __uint_as_float(v[j]) + __uint_as_float(u[j]);
      }
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&aempty[b]);
      const int64_t prob = 2 * pr + half;
      if (prob < g.batch && i < g.M) {
        float* cp = g.c + prob * g.stride_c + i + int64_t(c0) * g.ldc;
        const int nleft = g.N - c0;
        // C is read 16 columns at a time, all loads before any store, so the
        // loads overlap (a store may alias a later load when ldc == 0)
#pragma unroll
        for (int j0 = 0; j0 < 32; j0 += 16) {
          float cv[16];
          if (g.beta != 0.f) {
#pragma unroll
            for (int j = 0; j < 16; ++j) cv[j] = (j0 + j < nleft) ? cp[int64_t(j0 + j) * g.ldc] : 0.f;
          }
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            if (j0 + j < nleft) {
              float v = g.alpha * sum[j0 + j];
              if (g.beta != 0.f) v = fmaf(g.beta, cv[j], v);
              cp[int64_t(j0 + j) * g.ldc] = v;
            }
          }
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 2 * kBtAcc);
  }
}

// 3-D map over a strided batch of FP32 matrices: element (x, y) of matrix z
// at base[x + y*ld + z*stride], x < inner, y < outer; box 32 x box_outer x 1
// with the 128-byte swizzle.  False when TMA cannot address the layout.
static bool make_batch_map(CUtensorMap* map, const float* base, int64_t inner, int64_t outer, int64_t ld,
                           int64_t stride, int64_t batch, int box_outer) {
  EncodeTiledFn fn = tensor_map_encoder();
  if (!fn) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (ld * 4) % 16 || (stride * 4) % 16 || stride <= 0 || ld <= 0)
    return false;
  cuuint64_t dims[3] = {cuuint64_t(inner), cuuint64_t(outer), cuuint64_t(batch)};
  cuuint64_t strides[2] = {cuuint64_t(ld * 4), cuuint64_t(stride * 4)};
  cuuint32_t box[3] = {32, cuuint32_t(box_outer), 1};
  cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// UNSUPPORTED (nothing launched) when the batch does not suit this path.
gbblas_status_t launch_gemm_small_batched_tc(gbblas_handle_t h, const GemmArgs<float>& g) {
  if (g.m > 64 || g.n > 64 || g.k > 64 || g.k < 1 || g.batch < 2 || g.batch > (int64_t(1) << 31) ||
      g.alpha == 0.f)
    return GBBLAS_STATUS_UNSUPPORTED;
  // A(i, k): ta ? A[k + i*lda] : A[i + k*lda];  B(k, j): tb ? B[j + k*ldb] : B[k + j*ldb]
  CUtensorMap ma, mb;
  // operands that run along k: one 32 k x 64 row box per k-half; else two 32 x 32 boxes
  if (!make_batch_map(&ma, g.a, g.ta ? g.k : g.m, g.ta ? g.m : g.k, g.lda, g.stride_a, g.batch, g.ta ? 64 : 32) ||
      !make_batch_map(&mb, g.b, g.tb ? g.n : g.k, g.tb ? g.k : g.n, g.ldb, g.stride_b, g.batch, g.tb ? 32 : 64))
    return GBBLAS_STATUS_UNSUPPORTED;
  BtArgs a{int(g.m), int(g.n), int(g.k), g.batch, (g.batch + 1) / 2, g.alpha, g.beta, g.c, g.ldc, g.stride_c};
  const unsigned grid = unsigned(a.pairs < h->sm_count ? a.pairs : h->sm_count);
#define GB_BT(TA_, TB_)                                                                                        \
  if (g.ta == TA_ && g.tb == TB_) {                                                                            \
    static std::atomic<uint64_t> attr{0};                                                                      \
    GB_CUDA_TRY(raise_smem_limit(attr, reinterpret_cast<const void*>(batched_tc_kernel<TA_, TB_>), kBtSmem,    \
                                 h->device));                                                                  \
    batched_tc_kernel<TA_, TB_><<<grid, kBtThreads, kBtSmem, h->stream>>>(ma, mb, a, h->dev_error);            \
  }
  GB_BT(false, false)
  GB_BT(false, true)
  GB_BT(true, false)
  GB_BT(true, true)
#undef GB_BT
  return after_launch("batched_tc");
}

}  // namespace gb

// gemm_tc.cu — FP32 GEMM as split-BF16 products on the tcgen05 tensor cores.
//
// Each FP32 operand is split into P BF16 terms, x = x0 + x1 (+ x2), with
// x_{i+1} = bf16(x - x0 - ... - x_i) (exact residuals in FP32).  The product
// keeps the terms whose order is at least 2^-16 (P = 2: x0y0, x0y1, x1y0) or
// 2^-24 (P = 3: the six terms with i + j <= 2); every BF16 x BF16 product is
// exact and they accumulate in FP32, first in tensor memory per k-chunk, then
// in registers across chunks.
//
// Pipeline per CTA (128 x BN output tile, BK = 64):
//   warp 0      TMA producer: the P A-term tiles and P B-term tiles of one
//               k-block per stage (128-byte swizzle, K-major);
//   warp 1      allocates TMEM, one lane issues tcgen05.mma (M=128, K=16;
//               N=BN for each term pair when P <= 2; for P = 3 the six
//               products as four MMAs, two of them N=2*BN over the adjacent
//               B terms 0 and 1, into two column halves), commits each stage
//               back to the producer and each finished k-chunk accumulator
//               (two TMEM buffers) to the epilogue;
//   warps 2-5   epilogue: tcgen05.ld of each chunk into a per-thread FP32
//               row, then alpha/beta and stores to column-major C (beta == 0
//               never reads C).
// Every mbarrier wait is bounded; a wait that gives up records an error code
// in the handle's device error word and the CTA drains and frees TMEM.
//
// The split pre-pass writes the terms as [P][rows][Kp] BF16 (K contiguous,
// Kp = K rounded up to 64 with zeros), which also absorbs any transpose of A
// or B, so the tensor-core kernel only ever sees K-major operands.
#include <cuda_bf16.h>

#include <cstdlib>
#include <mutex>

#include "gemm_internal.cuh"
#include "selector.h"
#include "tc_ptx.cuh"

namespace gb {

constexpr int kTcBM = 128, kTcBK = 64, kTcThreads = 192;

template <int BN, int P, int STAGES>
struct TcCfg {
  static constexpr int A_TILE = kTcBM * kTcBK * 2;
  static constexpr int B_TILE = BN * kTcBK * 2;
  static constexpr int STAGE = P * (A_TILE + B_TILE);
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256;
  static constexpr int NPAIRS = P == 1 ? 1 : 3;  // term products issued one by one (P <= 2)
  // columns of one chunk accumulator: with P = 3 the products of an A term
  // with the two adjacent leading B terms are one N = 2*BN MMA, and the
  // epilogue adds the two column halves
  static constexpr int ACC = P == 3 ? 2 * BN : BN;
  static constexpr int TMEM_COLS = 2 * ACC;  // two chunk accumulators
  static_assert(SMEM <= 227 * 1024, "shared memory budget");
  static_assert(TMEM_COLS <= 512, "tensor memory budget");
};

// term pairs (a-term, b-term) of the P <= 2 splits, largest first:
// P = 1: (0,0); P = 2: (0,0) (0,1) (1,0)
__device__ __forceinline__ void term_pair(int q, int& pa, int& pb) {
  pa = q == 2 ? 1 : 0;
  pb = q == 1 ? 1 : 0;
}

// k-blocks (of 64) accumulated in tensor memory before the partial sum is
// promoted into the FP32 register accumulator of the epilogue warps
constexpr int kTcChunk = 4;


enum : int { kErrTcProducer = 101, kErrTcMma = 102, kErrTcEpilogue = 103, kErrTcDrain = 104 };

// Accumulation: the tensor core's FP32 accumulator is exact for each
// product but not correctly rounded when many products are summed, so the
// k loop is cut into chunks of kTcChunk k-blocks, each accumulated in its
// own TMEM buffer (two buffers, so the MMA warp runs one chunk ahead) and
// added by the epilogue warps into a per-thread FP32 register row.
// Batches and split-K slices run on gridDim.z (z = batch * split + slice);
// the operand terms of batch b are terms b*P .. b*P+P-1 of the tensor maps.
// PARTIAL: split-K slice — the raw tile goes to ws[batch][split][M][N].
constexpr int kTcGroupM = 16;  // 128-row tile rows per raster group (raster_m == 2)
template <int BN, int P, int STAGES, bool PARTIAL>
__global__ void __launch_bounds__(kTcThreads, 1)
    gemm_split_bf16_kernel(const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_b,
                           int M, int N, int nk_total, int split, int kb_per_split, float alpha, float beta,
                           float* __restrict__ C, int64_t ldc, int64_t stride_c, float* __restrict__ ws,
                           int raster_m, int* __restrict__ err) {
  using Cfg = TcCfg<BN, P, STAGES>;
  const int bz = blockIdx.z / split, slice = blockIdx.z % split;
  const int kb0 = slice * kb_per_split;
  const int nk = max(0, min(nk_total - kb0, kb_per_split));
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* tiles = smem;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * Cfg::STAGE);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;  // [2] chunk accumulator ready
  uint64_t* tempty = tfull + 2;      // [2] chunk accumulator drained
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // raster_m 1: consecutive CTAs walk down M (share a B tile) instead of
  // along N; 2: grid (N tiles, M tiles) taken in groups of kTcGroupM tile
  // rows, down M within a group, so the CTAs resident together share A and
  // B panels in L2 when neither operand fits there
  int mt, ntile;
  if (raster_m == 2) {
    const int lin = int(blockIdx.y * gridDim.x + blockIdx.x), tn = int(gridDim.x), tm = int(gridDim.y);
    const int first = (lin / (kTcGroupM * tn)) * kTcGroupM, in = lin % (kTcGroupM * tn);
    const int gsize = min(tm - first, kTcGroupM);
    mt = first + in % gsize;
    ntile = in / gsize;
  } else {
    mt = raster_m ? blockIdx.x : blockIdx.y;
    ntile = raster_m ? blockIdx.y : blockIdx.x;
  }
  const int m0 = mt * kTcBM;
  const int n0 = ntile * BN;
  const int nchunks = (nk + kTcChunk - 1) / kTcChunk;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&tfull[b], 1);
      tc::mbar_init(&tempty[b], 4);  // one arrival per epilogue warp
    }
    tc::fence_mbar_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tmem_slot, Cfg::TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  pdl_wait();  // the operand terms (and C) are written by earlier kernels on the stream

  if (warp == 0) {
    if (lane == 0) {
      tc::tma_prefetch_desc(&tma_a);
      tc::tma_prefetch_desc(&tma_b);
      int issued = 0;
      for (int kb = 0; kb < nk; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!tc::mbar_wait(&empty[s], ph ^ 1)) {
          atomicExch(err, kErrTcProducer);
          break;
        }
        tc::mbar_arrive_expect_tx(&full[s], Cfg::STAGE);
        uint8_t* st = tiles + s * Cfg::STAGE;
#pragma unroll
        for (int p = 0; p < P; ++p)
          tc::tma_load_3d(st + p * Cfg::A_TILE, &tma_a, &full[s], (kb0 + kb) * kTcBK, m0, bz * P + p);
#pragma unroll
        for (int p = 0; p < P; ++p)
          tc::tma_load_3d(st + P * Cfg::A_TILE + p * Cfg::B_TILE, &tma_b, &full[s], (kb0 + kb) * kTcBK, n0,
                          bz * P + p);
        issued = kb + 1;
      }
      // drain: every copy this thread issued has landed before the CTA exits
      for (int kb = issued > STAGES ? issued - STAGES : 0; kb < issued; ++kb)
        if (!tc::mbar_wait(&full[kb % STAGES], (kb / STAGES) & 1)) {
          atomicExch(err, kErrTcDrain);
          break;
        }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(kTcBM, BN);
      constexpr uint32_t idesc2 = tc::idesc_bf16_f32(kTcBM, 2 * BN);
      bool ok = true;
      for (int c = 0; c < nchunks && ok; ++c) {
        const int b = c & 1;
        if (!tc::mbar_wait(&tempty[b], ((c >> 1) & 1) ^ 1)) {
          atomicExch(err, kErrTcMma);
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const uint32_t acc = tmem + uint32_t(b * Cfg::ACC);
        const int kb1 = min(nk, (c + 1) * kTcChunk);
        for (int kb = c * kTcChunk; kb < kb1; ++kb) {
          const int s = kb % STAGES;
          const uint32_t ph = (kb / STAGES) & 1;
          if (!tc::mbar_wait(&full[s], ph)) {
            atomicExch(err, kErrTcMma);
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint8_t* st = tiles + s * Cfg::STAGE;
          if constexpr (P <= 2) {
#pragma unroll
            for (int q = 0; q < Cfg::NPAIRS; ++q) {
              int pa, pb;
              term_pair(q, pa, pb);
              const uint64_t ad = tc::sdesc_kmajor_sw128(tc::smem_u32(st + pa * Cfg::A_TILE));
              const uint64_t bd = tc::sdesc_kmajor_sw128(tc::smem_u32(st + P * Cfg::A_TILE + pb * Cfg::B_TILE));
#pragma unroll
              for (int j = 0; j < kTcBK / 16; ++j)  // K = 16 per MMA: +32 bytes in the swizzled row
                tc::mma_bf16(acc, ad + 2 * j, bd + 2 * j, idesc, (kb != c * kTcChunk) || q != 0 || j != 0);
            }
          } else {
            // P = 3: the B terms are adjacent BN-row tiles, so B terms (0, 1)
            // form one 2*BN-row operand.  a(0) x [b0; b1] fills both column
            // halves (the first MMA of a chunk initialises both), a(1) x
            // [b0; b1] adds to both, a(0) b(2) and a(2) b(0) go to the second
            // half: the six products of the split, the leading one kept apart
            // from the small cross terms.
            const uint32_t sa = tc::smem_u32(st), sb = tc::smem_u32(st + P * Cfg::A_TILE);
            const uint64_t a0 = tc::sdesc_kmajor_sw128(sa), a1 = tc::sdesc_kmajor_sw128(sa + Cfg::A_TILE);
            const uint64_t a2 = tc::sdesc_kmajor_sw128(sa + 2 * Cfg::A_TILE);
            const uint64_t b01 = tc::sdesc_kmajor_sw128(sb), b2 = tc::sdesc_kmajor_sw128(sb + 2 * Cfg::B_TILE);
            const uint32_t acc2 = acc + uint32_t(BN);
#pragma unroll
            for (int j = 0; j < kTcBK / 16; ++j) {  // K = 16 per MMA: +32 bytes in the swizzled row
              tc::mma_bf16(acc, a0 + 2 * j, b01 + 2 * j, idesc2, (kb != c * kTcChunk) || j != 0);
              tc::mma_bf16(acc, a1 + 2 * j, b01 + 2 * j, idesc2, true);
              tc::mma_bf16(acc2, a0 + 2 * j, b2 + 2 * j, idesc, true);
              tc::mma_bf16(acc2, a2 + 2 * j, b01 + 2 * j, idesc, true);
            }
          }
          tc::mma_commit(&empty[s]);
        }
        if (ok) tc::mma_commit(&tfull[b]);
      }
    }
  } else {
    // epilogue warps 2..5: warp w owns TMEM lanes [32*(w%4), 32*(w%4)+32),
    // i.e. one output row per thread, all BN columns in registers
    const int q = warp & 3;
    const int row = q * 32 + lane;
    const int gm = m0 + row;
    float sum[BN];
#pragma unroll
    for (int i = 0; i < BN; ++i) sum[i] = 0.f;
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
      const int b = c & 1;
      if (!tc::mbar_wait(&tfull[b], (c >> 1) & 1)) {
        if (lane == 0) atomicExch(err, kErrTcEpilogue);
        ok = false;
        break;
      }
      tc::tc_fence_after();
#pragma unroll
      for (int c0 = 0; c0 < Cfg::ACC; c0 += 32) {  // column halves fold onto the same BN sums
        uint32_t r[32];
        tc::tmem_ld_32x32b_x32(tmem + (uint32_t(q * 32) << 16) + uint32_t(b * Cfg::ACC + c0), r);
        tc::tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 32; ++i) sum[(c0 + i) % BN] += __uint_as_float(r[i]);
      }
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&tempty[b]);
    }
    if (ok && gm < M) {
      if (PARTIAL) {
        float* W0 = ws + (int64_t(bz) * split + slice) * int64_t(M) * N;
#pragma unroll
        for (int i = 0; i < BN; ++i) {
          const int gn = n0 + i;
          if (gn < N) W0[int64_t(gm) + int64_t(gn) * M] = sum[i];
        }
      } else {
        // C is read 32 columns at a time, all loads before any store, so the
        // loads overlap (a store may alias a later load when ldc == 0, so the
        // compiler cannot reorder them itself); beta == 0 never reads C
        float* rowp = C + int64_t(bz) * stride_c + int64_t(gm);
#pragma unroll
        for (int g0 = 0; g0 < BN; g0 += 32) {
          float cv[32];
          if (beta != 0.f) {
#pragma unroll
            for (int i = 0; i < 32; ++i) cv[i] = (n0 + g0 + i < N) ? rowp[int64_t(n0 + g0 + i) * ldc] : 0.f;
          }
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int gn = n0 + g0 + i;
            if (gn < N) {
              float v = alpha * sum[g0 + i];
              if (beta != 0.f) v = fmaf(beta, cv[i], v);
              rowp[int64_t(gn) * ldc] = v;
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
    tc::tmem_dealloc(tmem, Cfg::TMEM_COLS);
  }
}

// ---------------------------------------------------- CTA-pair (2-SM) tiles --
// The 2-term split (x3) on 256 x 128 output tiles, one at a time per cluster
// of two CTAs: each CTA loads its own 128 rows of A and half (64 rows) of the
// B tile, so a stage is 48 KB instead of 64 and four fit; the even CTA's MMA
// lane issues tcgen05.mma.cta_group::2 (M = 256: A rows 0..127 from the even
// CTA, 128..255 from the odd one; B columns 0..63 from the even CTA, 64..127
// from the odd one), so each SM's tensor core reads half of B from shared
// memory.  Both CTAs' TMA loads count on the even CTA's full barrier; its
// commits arrive on both CTAs' stage-free and chunk-ready barriers; both
// CTAs' eight epilogue warps drain their own 128 rows of TMEM (four chunk
// accumulators) and arrive on the even CTA's chunk-free barrier.
// Persistent: the grid is the clusters that can be resident at once, and
// cluster c takes tiles c, c + clusters, ... of a fixed order (batch, then
// groups of kPairGroupM 256-row tile rows down M, then along N, so the
// clusters working at the same time share A and B panels in L2).  Stage and
// chunk counters run on across tiles, so the MMAs of the next tile fill the
// free accumulators while the epilogue stores C, and the ring never drains
// at a tile boundary.  Every mbarrier wait is bounded; the two CTAs meet in
// cluster barriers only after setup and before TMEM is freed.
constexpr int kPairBN = 128, kPairBHalf = kPairBN / 2;
// warps: 0 producer, 1 MMA (even CTA), 2..9 epilogue (two per TMEM lane quarter, 64 columns each)
constexpr int kPairEpiWarps = 8, kPairThreads = 32 * (2 + kPairEpiWarps);
constexpr int kPairAcc = 4;     // chunk accumulators in TMEM (the MMAs run up to three chunks ahead)
constexpr int kPairGroupM = 8;  // 256-row tile rows per raster group

template <int STAGES>
struct PairCfg {
  static constexpr int P = 2;
  static constexpr int A_TILE = kTcBM * kTcBK * 2;     // 16 KB
  static constexpr int B_TILE = kPairBHalf * kTcBK * 2;  // 8 KB
  static constexpr int STAGE = P * (A_TILE + B_TILE);  // 48 KB
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256;
  static constexpr int TMEM_COLS = kPairAcc * kPairBN;  // all 512 columns
  static_assert(SMEM <= 227 * 1024, "shared memory budget");
};

// Tile t of the fixed order: batch bz, 256-row tile row mp, 128-column tile nt.
__device__ __forceinline__ void pair_tile(int t, int mp_count, int nt_count, int& bz, int& mp, int& nt) {
  const int per_batch = mp_count * nt_count;
  bz = t / per_batch;
  const int r = t - bz * per_batch;
  const int per_group = kPairGroupM * nt_count;
  const int first = (r / per_group) * kPairGroupM, in = r % per_group;
  const int gsize = min(mp_count - first, kPairGroupM);
  mp = first + in % gsize;
  nt = in / gsize;
}

enum : int { kErrPairProducer = 111, kErrPairMma = 112, kErrPairEpilogue = 113, kErrPairDrain = 114 };

template <int STAGES>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kPairThreads, 1)
    gemm_split_bf16_pair_kernel(const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_b,
                                int M, int N, int nk, int tiles, float alpha, float beta, float* __restrict__ C,
                                int64_t ldc, int64_t stride_c, int* __restrict__ err) {
  using Cfg = PairCfg<STAGES>;
  constexpr int P = Cfg::P;
  const uint32_t rank = tc::cluster_ctarank();  // 0: issues the MMAs
  const int cid = int(blockIdx.x >> 1), clusters = int(gridDim.x >> 1);
  const int mp_count = (M + 2 * kTcBM - 1) / (2 * kTcBM), nt_count = (N + kPairBN - 1) / kPairBN;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* tiles_smem = smem;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * Cfg::STAGE);  // even CTA: both CTAs' bytes
  uint64_t* empty = full + STAGES;   // both CTAs: the MMAs that read the stage are done
  uint64_t* tfull = empty + STAGES;      // [kPairAcc] both CTAs: chunk accumulator ready
  uint64_t* tempty = tfull + kPairAcc;   // [kPairAcc] even CTA: chunk drained by both CTAs' epilogues
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + kPairAcc);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunks = (nk + kTcChunk - 1) / kTcChunk;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < kPairAcc; ++b) {
      tc::mbar_init(&tfull[b], 1);
      tc::mbar_init(&tempty[b], 2 * kPairEpiWarps);  // the epilogue warps of both CTAs
    }
    tc::fence_mbar_init();
  }
  if (warp == 1) {
    tc::tmem_alloc_pair(tmem_slot, Cfg::TMEM_COLS);
    tc::tmem_relinquish_pair();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::cluster_sync();  // the peer's barriers are initialised before anything targets them
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  pdl_wait();  // the operand terms (and C) are written by earlier kernels on the stream

  if (warp == 0) {
    if (lane == 0) {
      tc::tma_prefetch_desc(&tma_a);
      tc::tma_prefetch_desc(&tma_b);
      const uint32_t full0 = tc::mapa_shared(tc::smem_u32(full), 0);
      uint32_t it = 0;  // k-blocks issued, over all tiles
      bool ok = true;
      for (int t = cid; t < tiles && ok; t += clusters) {
        int bz, mp, nt;
        pair_tile(t, mp_count, nt_count, bz, mp, nt);
        const int m0 = mp * (2 * kTcBM) + int(rank) * kTcBM, n0 = nt * kPairBN;
        for (int kb = 0; kb < nk; ++kb, ++it) {
          const int s = int(it % STAGES);
          if (!tc::mbar_wait(&empty[s], ((it / STAGES) & 1) ^ 1)) {
            atomicExch(err, kErrPairProducer);
            ok = false;
            break;
          }
          if (rank == 0) tc::mbar_arrive_expect_tx(&full[s], 2 * Cfg::STAGE);
          const uint32_t bar = full0 + uint32_t(s) * 8u;
          uint8_t* st = tiles_smem + s * Cfg::STAGE;
#pragma unroll
          for (int p = 0; p < P; ++p)
            tc::tma_load_3d_pair(st + p * Cfg::A_TILE, &tma_a, bar, kb * kTcBK, m0, bz * P + p);
#pragma unroll
          for (int p = 0; p < P; ++p)
            tc::tma_load_3d_pair(st + P * Cfg::A_TILE + p * Cfg::B_TILE, &tma_b, bar, kb * kTcBK,
                                 n0 + int(rank) * kPairBHalf, bz * P + p);
        }
      }
      // drain (even CTA): every copy of the pair has landed before the CTA exits
      if (rank == 0)
        for (uint32_t j = it > uint32_t(STAGES) ? it - STAGES : 0u; j < it; ++j)
          if (!tc::mbar_wait(&full[j % STAGES], (j / STAGES) & 1)) {
            atomicExch(err, kErrPairDrain);
            break;
          }
    }
  } else if (warp == 1) {
    if (lane == 0 && rank == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(2 * kTcBM, kPairBN);
      uint32_t it = 0, g = 0;  // k-blocks and chunks consumed, over all tiles
      bool ok = true;
      for (int t = cid; t < tiles && ok; t += clusters) {
        for (int c = 0; c < nchunks && ok; ++c, ++g) {
          const int b = int(g % kPairAcc);
          if (!tc::mbar_wait(&tempty[b], ((g / kPairAcc) & 1) ^ 1)) {
            atomicExch(err, kErrPairMma);
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t acc = tmem + uint32_t(b * kPairBN);
          const int kb1 = min(nk, (c + 1) * kTcChunk);
          for (int kb = c * kTcChunk; kb < kb1; ++kb, ++it) {
            const int s = int(it % STAGES);
            if (!tc::mbar_wait(&full[s], (it / STAGES) & 1)) {
              atomicExch(err, kErrPairMma);
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint8_t* st = tiles_smem + s * Cfg::STAGE;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
              int pa, pb;
              term_pair(q, pa, pb);
              const uint64_t ad = tc::sdesc_kmajor_sw128(tc::smem_u32(st + pa * Cfg::A_TILE));
              const uint64_t bd = tc::sdesc_kmajor_sw128(tc::smem_u32(st + P * Cfg::A_TILE + pb * Cfg::B_TILE));
#pragma unroll
              for (int j = 0; j < kTcBK / 16; ++j)
                tc::mma_bf16_pair(acc, ad + 2 * j, bd + 2 * j, idesc, (kb != c * kTcChunk) || q != 0 || j != 0);
            }
            tc::mma_commit_pair(&empty[s], 0x3);
          }
          if (ok) tc::mma_commit_pair(&tfull[b], 0x3);
        }
      }
    }
  } else {
    // epilogue warps 2..9: warp w owns TMEM lanes [32*(w%4), +32) (one row of
    // this CTA's 128 per thread) and columns [64*h, +64), h = (w - 2) / 4
    const int q = warp & 3, h = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const uint32_t tempty0 = tc::mapa_shared(tc::smem_u32(tempty), 0);
    uint32_t g = 0;  // chunks drained, over all tiles
    bool ok = true;
    for (int t = cid; t < tiles && ok; t += clusters) {
      int bz, mp, nt;
      pair_tile(t, mp_count, nt_count, bz, mp, nt);
      const int gm = mp * (2 * kTcBM) + int(rank) * kTcBM + row, n0 = nt * kPairBN;
      float sum[64];
#pragma unroll
      for (int i = 0; i < 64; ++i) sum[i] = 0.f;
      for (int c = 0; c < nchunks; ++c, ++g) {
        const int b = int(g % kPairAcc);
        if (!tc::mbar_wait(&tfull[b], (g / kPairAcc) & 1)) {
          if (lane == 0) atomicExch(err, kErrPairEpilogue);
          ok = false;
          break;
        }
        tc::tc_fence_after();
        uint32_t r0[32], r1[32];
        const uint32_t base = tmem + (uint32_t(q * 32) << 16) + uint32_t(b * kPairBN + h * 64);
        tc::tmem_ld_32x32b_x32(base, r0);
        tc::tmem_ld_32x32b_x32(base + 32u, r1);
        tc::tmem_ld_wait();
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          sum[i] += __uint_as_float(r0[i]);
          sum[32 + i] += __uint_as_float(r1[i]);
        }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive_cluster(tempty0 + uint32_t(b) * 8u);
      }
      if (ok && gm < M) {
        float* rowp = C + int64_t(bz) * stride_c + int64_t(gm);
        const int nb = n0 + h * 64;
#pragma unroll
        for (int g0 = 0; g0 < 64; g0 += 32) {
          float cv[32];
          if (beta != 0.f) {
#pragma unroll
            for (int i = 0; i < 32; ++i) cv[i] = (nb + g0 + i < N) ? rowp[int64_t(nb + g0 + i) * ldc] : 0.f;
          }
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int gn = nb + g0 + i;
            if (gn < N) {
              float v = alpha * sum[g0 + i];
              if (beta != 0.f) v = fmaf(beta, cv[i], v);
              rowp[int64_t(gn) * ldc] = v;
            }
          }
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::cluster_sync();  // both CTAs are done with each other's barriers and shared memory
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc_pair(tmem, Cfg::TMEM_COLS);
  }
}

// ------------------------------------------- CTA-pair tiles of 256 x 256 --
// The same schedule as the 256 x 128 pair kernel above with N = 256 per
// cluster: each CTA loads its 128 rows of A and 128 rows (its half) of B per
// term and stage (x3: 64 KB, three stages; x6: 96 KB, two stages), the even
// CTA issues tcgen05.mma.cta_group::2 M256 N256 K16, so each MMA does twice
// the work for the same A read; every term product of a TMEM chunk goes into
// one accumulator (two of 256 columns, so the MMAs of the next chunk run
// while the epilogue promotes this one); sixteen epilogue warps per CTA, four
// per TMEM lane quarter, each with 64 of the 256 columns.  A short last
// round (at most half the clusters) runs as 256 x 128 halves of its tiles
// (pair2_item): each CTA loads 64 B rows through a second tensor map, the
// MMA is N = 128 and the epilogue warps past column 128 store nothing.
// Used where the 256 x 256 tiles fill at least half of the resident
// clusters.
constexpr int kPair2BN = 256, kPair2BHalf = kPair2BN / 2;
constexpr int kPair2EpiWarps = 16, kPair2Threads = 32 * (2 + kPair2EpiWarps);
constexpr int kPair2Acc = 2;

template <int P_, int STAGES>
struct Pair2Cfg {
  static constexpr int P = P_;
  static constexpr int A_TILE = kTcBM * kTcBK * 2;        // 16 KB
  static constexpr int B_TILE = kPair2BHalf * kTcBK * 2;  // 16 KB
  static constexpr int STAGE = P * (A_TILE + B_TILE);     // 64 KB (x3) / 96 KB (x6)
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256;
  static constexpr int TMEM_COLS = kPair2Acc * kPair2BN;  // all 512 columns
  // term products per k-block: x3 (0,0) (0,1) (1,0); x6 adds (1,1) (0,2) (2,0)
  static constexpr int NPROD = P == 2 ? 3 : 6;
  // k-blocks per TMEM chunk: every product of the chunk goes into the one
  // accumulator, so x6 (six MMAs per K16 step) promotes twice as often
  static constexpr int CHUNK = P == 2 ? kTcChunk : kTcChunk / 4;
  static_assert(SMEM <= 227 * 1024, "shared memory budget");
};

// (a-term, b-term) of product q, largest first
__device__ __forceinline__ void term_pair6(int q, int& pa, int& pb) {
  constexpr int kA[6] = {0, 0, 1, 1, 0, 2}, kB[6] = {0, 1, 0, 1, 2, 0};
  pa = kA[q];
  pb = kB[q];
}

// Work item t of the persistent loop: items below `full` (whole rounds of
// the clusters) are 256 x 256 tiles in pair_tile order; the items after
// them are the two 256 x 128 halves of each remaining tile, so a short last
// round is spread over twice as many clusters at half the work each.
struct Pair2Item {
  int bz, mp, n0, width;
};
__device__ __forceinline__ Pair2Item pair2_item(int t, int whole, int mp_count, int nt_count) {
  Pair2Item w;
  const bool half = t >= whole;
  const int tt = half ? whole + ((t - whole) >> 1) : t;
  int nt;
  pair_tile(tt, mp_count, nt_count, w.bz, w.mp, nt);
  w.width = half ? kPair2BHalf : kPair2BN;
  w.n0 = nt * kPair2BN + (half ? ((t - whole) & 1) * kPair2BHalf : 0);
  return w;
}

template <int P, int STAGES>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kPair2Threads, 1)
    gemm_split_bf16_pair256_kernel(const __grid_constant__ CUtensorMap tma_a,
                                   const __grid_constant__ CUtensorMap tma_b,
                                   const __grid_constant__ CUtensorMap tma_b_half, int M, int N, int nk, int whole,
                                   int items, float alpha, float beta, float* __restrict__ C, int64_t ldc,
                                   int64_t stride_c, int* __restrict__ err) {
  using Cfg = Pair2Cfg<P, STAGES>;
  const uint32_t rank = tc::cluster_ctarank();  // 0: issues the MMAs
  const int cid = int(blockIdx.x >> 1), clusters = int(gridDim.x >> 1);
  const int mp_count = (M + 2 * kTcBM - 1) / (2 * kTcBM), nt_count = (N + kPair2BN - 1) / kPair2BN;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* tiles_smem = smem;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * Cfg::STAGE);  // even CTA: both CTAs' bytes
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;      // [kPair2Acc]
  uint64_t* tempty = tfull + kPair2Acc;  // [kPair2Acc] even CTA: drained by both CTAs' epilogues
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + kPair2Acc);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunks = (nk + Cfg::CHUNK - 1) / Cfg::CHUNK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < kPair2Acc; ++b) {
      tc::mbar_init(&tfull[b], 1);
      tc::mbar_init(&tempty[b], 2 * kPair2EpiWarps);  // the epilogue warps of both CTAs
    }
    tc::fence_mbar_init();
  }
  if (warp == 1) {
    tc::tmem_alloc_pair(tmem_slot, Cfg::TMEM_COLS);
    tc::tmem_relinquish_pair();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::cluster_sync();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  pdl_wait();  // the operand terms (and C) are written by earlier kernels on the stream

  if (warp == 0) {
    if (lane == 0) {
      tc::tma_prefetch_desc(&tma_a);
      tc::tma_prefetch_desc(&tma_b);
      const uint32_t full0 = tc::mapa_shared(tc::smem_u32(full), 0);
      uint32_t it = 0;
      bool ok = true;
      for (int t = cid; t < items && ok; t += clusters) {
        const Pair2Item w = pair2_item(t, whole, mp_count, nt_count);
        const bool narrow = w.width < kPair2BN;  // this CTA loads w.width / 2 B rows
        const int m0 = w.mp * (2 * kTcBM) + int(rank) * kTcBM, n0 = w.n0 + int(rank) * (w.width / 2);
        const uint32_t bytes = 2u * uint32_t(P * (Cfg::A_TILE + (narrow ? Cfg::B_TILE / 2 : Cfg::B_TILE)));
        for (int kb = 0; kb < nk; ++kb, ++it) {
          const int s = int(it % STAGES);
          if (!tc::mbar_wait(&empty[s], ((it / STAGES) & 1) ^ 1)) {
            atomicExch(err, kErrPairProducer);
            ok = false;
            break;
          }
          if (rank == 0) tc::mbar_arrive_expect_tx(&full[s], bytes);
          const uint32_t bar = full0 + uint32_t(s) * 8u;
          uint8_t* st = tiles_smem + s * Cfg::STAGE;
#pragma unroll
          for (int p = 0; p < P; ++p)
            tc::tma_load_3d_pair(st + p * Cfg::A_TILE, &tma_a, bar, kb * kTcBK, m0, w.bz * P + p);
#pragma unroll
          for (int p = 0; p < P; ++p)
            tc::tma_load_3d_pair(st + P * Cfg::A_TILE + p * Cfg::B_TILE, narrow ? &tma_b_half : &tma_b, bar,
                                 kb * kTcBK, n0, w.bz * P + p);
        }
      }
      if (rank == 0)
        for (uint32_t j = it > uint32_t(STAGES) ? it - STAGES : 0u; j < it; ++j)
          if (!tc::mbar_wait(&full[j % STAGES], (j / STAGES) & 1)) {
            atomicExch(err, kErrPairDrain);
            break;
          }
    }
  } else if (warp == 1) {
    if (lane == 0 && rank == 0) {
      uint32_t it = 0, g = 0;
      bool ok = true;
      for (int t = cid; t < items && ok; t += clusters) {
        const uint32_t idesc = tc::idesc_bf16_f32(2 * kTcBM, t < whole ? kPair2BN : kPair2BHalf);
        for (int c = 0; c < nchunks && ok; ++c, ++g) {
          const int b = int(g % kPair2Acc);
          if (!tc::mbar_wait(&tempty[b], ((g / kPair2Acc) & 1) ^ 1)) {
            atomicExch(err, kErrPairMma);
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t acc = tmem + uint32_t(b * kPair2BN);
          const int kb1 = min(nk, (c + 1) * Cfg::CHUNK);
          for (int kb = c * Cfg::CHUNK; kb < kb1; ++kb, ++it) {
            const int s = int(it % STAGES);
            if (!tc::mbar_wait(&full[s], (it / STAGES) & 1)) {
              atomicExch(err, kErrPairMma);
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint8_t* st = tiles_smem + s * Cfg::STAGE;
#pragma unroll
            for (int q = 0; q < Cfg::NPROD; ++q) {
              int pa, pb;
              term_pair6(q, pa, pb);
              const uint64_t ad = tc::sdesc_kmajor_sw128(tc::smem_u32(st + pa * Cfg::A_TILE));
              const uint64_t bd = tc::sdesc_kmajor_sw128(tc::smem_u32(st + P * Cfg::A_TILE + pb * Cfg::B_TILE));
#pragma unroll
              for (int j = 0; j < kTcBK / 16; ++j)
                tc::mma_bf16_pair(acc, ad + 2 * j, bd + 2 * j, idesc, (kb != c * Cfg::CHUNK) || q != 0 || j != 0);
            }
            tc::mma_commit_pair(&empty[s], 0x3);
          }
          if (ok) tc::mma_commit_pair(&tfull[b], 0x3);
        }
      }
    }
  } else {
    // epilogue warps 2..17: warp w owns TMEM lanes [32*(w%4), +32) (one row
    // of this CTA's 128 per thread) and columns [64*cg, +64), cg = (w - 2) / 4
    const int q = warp & 3, cg = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const uint32_t tempty0 = tc::mapa_shared(tc::smem_u32(tempty), 0);
    uint32_t g = 0;
    bool ok = true;
    for (int t = cid; t < items && ok; t += clusters) {
      const Pair2Item w = pair2_item(t, whole, mp_count, nt_count);
      const int bz = w.bz;
      const int gm = w.mp * (2 * kTcBM) + int(rank) * kTcBM + row, nb = w.n0 + cg * 64;
      // a half-width item's accumulator holds 128 columns: warps past them
      // drain their share and store nothing
      const bool cols_in = cg * 64 < w.width;
      float sum[64];
#pragma unroll
      for (int i = 0; i < 64; ++i) sum[i] = 0.f;
      for (int c = 0; c < nchunks; ++c, ++g) {
        const int b = int(g % kPair2Acc);
        if (!tc::mbar_wait(&tfull[b], (g / kPair2Acc) & 1)) {
          if (lane == 0) atomicExch(err, kErrPairEpilogue);
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const uint32_t base = tmem + (uint32_t(q * 32) << 16) + uint32_t(b * kPair2BN + cg * 64);
        // 8 columns per wait: the 64 running sums and the loaded values fit
        // the 96 registers a thread of an 18-warp CTA gets
#pragma unroll
        for (int hh = 0; hh < 8; ++hh) {
          uint32_t r0[8];
          tc::tmem_ld_32x32b_x8(base + uint32_t(8 * hh), r0);
          tc::tmem_ld_wait();
#pragma unroll
          for (int i = 0; i < 8; ++i) sum[8 * hh + i] += __uint_as_float(r0[i]);
        }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive_cluster(tempty0 + uint32_t(b) * 8u);
      }
      if (ok && gm < M && cols_in) {
        float* rowp = C + int64_t(bz) * stride_c + int64_t(gm);
#pragma unroll
        for (int g0 = 0; g0 < 64; g0 += 8) {
          float cv[8];
          if (beta != 0.f) {
#pragma unroll
            for (int i = 0; i < 8; ++i) cv[i] = (nb + g0 + i < N) ? rowp[int64_t(nb + g0 + i) * ldc] : 0.f;
          }
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int gn = nb + g0 + i;
            if (gn < N) {
              float v = alpha * sum[g0 + i];
              if (beta != 0.f) v = fmaf(beta, cv[i], v);
              rowp[int64_t(gn) * ldc] = v;
            }
          }
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::cluster_sync();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc_pair(tmem, Cfg::TMEM_COLS);
  }
}

// ------------------------------------------------------------ split pass --
// out[p][r][k] (k < Kp) = term p of X(r, k); X(r, k) = X[r*sr + k*sk]; zero
// for k >= K; Kp is a multiple of 64.  One CTA per 64 x 64 tile, 256
// threads; thread t writes the eight k from 8 (t % 8) of rows t / 8 and
// t / 8 + 32 of the tile, one 16-byte store per row and term.  K-contiguous
// operands (sk == 1) are read straight into registers (two 16-byte loads per
// row when rows are 16-byte aligned); others are transposed through shared
// memory, each thread with 16 loads in flight along the contiguous rows.
// One operand of the split pass (A or B of the GEMM).
struct SplitOperand {
  const float* X;
  int64_t sr, sk, R, xstride;
  int vec4;  // sk == 1 with 16-byte-aligned rows
  __nv_bfloat16* out;
};

// Both operands in one launch: blockIdx.z = 2 * batch + operand; tiles past
// an operand's rows exit at once.
template <int P>
__global__ void __launch_bounds__(256) split_bf16_kernel(SplitOperand a, SplitOperand b, int64_t K, int64_t Kp) {
  pdl_trigger();  // the GEMM that reads the terms may place its CTAs and set up meanwhile
  __shared__ float t[64][65];  // t[k][r]
  const SplitOperand& op = (blockIdx.z & 1) ? b : a;
  const int64_t R = op.R, sr = op.sr, sk = op.sk;
  const int vec4 = op.vec4;
  const int64_t r0 = int64_t(blockIdx.y) * 64, k0 = int64_t(blockIdx.x) * 64;
  if (r0 >= R) return;
  const float* __restrict__ X = op.X + int64_t(blockIdx.z >> 1) * op.xstride;
  __nv_bfloat16* __restrict__ out = op.out + int64_t(blockIdx.z >> 1) * P * R * Kp;
  const int tid = threadIdx.x, c = tid & 7;
  const int64_t k = k0 + 8 * c;
  float x[2][8];
  if (sk == 1) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t r = r0 + (tid >> 3) + 32 * h;
      const float* q = X + r * sr + k;
      if (r < R && vec4 && k + 8 <= K) {
        const float4 a = __ldcs(reinterpret_cast<const float4*>(q));
        const float4 b = __ldcs(reinterpret_cast<const float4*>(q + 4));
        x[h][0] = a.x; x[h][1] = a.y; x[h][2] = a.z; x[h][3] = a.w;
        x[h][4] = b.x; x[h][5] = b.y; x[h][6] = b.z; x[h][7] = b.w;
      } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) x[h][e] = (r < R && k + e < K) ? __ldcs(q + e) : 0.f;
      }
    }
  } else {
    const int rr = tid & 63, kq = tid >> 6;
    const bool rok = r0 + rr < R;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int64_t kk = k0 + kq + 4 * i;
      t[kq + 4 * i][rr] = (rok && kk < K) ? __ldcs(X + (r0 + rr) * sr + kk * sk) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int e = 0; e < 8; ++e) x[h][e] = t[8 * c + e][(tid >> 3) + 32 * h];
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int64_t r = r0 + (tid >> 3) + 32 * h;
    if (r >= R) continue;
    __nv_bfloat16* o = out + r * Kp + k;
#pragma unroll
    for (int p = 0; p < P; ++p) {
      uint32_t w[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const __nv_bfloat162 h2 = __floats2bfloat162_rn(x[h][2 * e], x[h][2 * e + 1]);
        w[e] = *reinterpret_cast<const uint32_t*>(&h2);
        x[h][2 * e] -= __uint_as_float(w[e] << 16);  // exact residuals
        x[h][2 * e + 1] -= __uint_as_float(w[e] & 0xffff0000u);
      }
      // plain stores: a small GEMM finds its terms still in L2
      *reinterpret_cast<uint4*>(o + int64_t(p) * R * Kp) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

// ------------------------------------------------------------------ host --
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn tensor_map_encoder() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// [P][rows][Kp] BF16 terms, box = 64 (k) x box_rows x 1
static gbblas_status_t make_term_map(CUtensorMap* map, void* base, int64_t rows, int64_t Kp, int P, int box_rows) {
  EncodeTiledFn fn = tensor_map_encoder();
  if (!fn) return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {cuuint64_t(Kp), cuuint64_t(rows), cuuint64_t(P)};
  cuuint64_t strides[2] = {cuuint64_t(Kp * 2), cuuint64_t(rows * Kp * 2)};
  cuuint32_t box[3] = {cuuint32_t(kTcBK), cuuint32_t(box_rows), 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: tensor map encode failed (" + std::to_string(int(r)) + ")");
  return GBBLAS_STATUS_SUCCESS;
}

static SplitOperand split_operand(const float* X, int64_t sr, int64_t sk, int64_t R, int64_t xstride,
                                  __nv_bfloat16* out) {
  const int vec4 = sk == 1 && sr % 4 == 0 && xstride % 4 == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0;
  return SplitOperand{X, sr, sk, R, xstride, vec4, out};
}

// The terms of A and B, one launch.
template <int P>
static gbblas_status_t launch_split(gbblas_handle_t h, const SplitOperand& a, const SplitOperand& b, int64_t K,
                                    int64_t Kp, int64_t batch) {
  const int64_t rt = cdiv(a.R > b.R ? a.R : b.R, 64);
  if (rt > 65535) return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: grid too large");
  constexpr int64_t kMaxBatch = 65535 / 2;  // grid z = 2 per batch entry
  for (int64_t b0 = 0; b0 < batch; b0 += kMaxBatch) {
    const int64_t nb = batch - b0 < kMaxBatch ? batch - b0 : kMaxBatch;
    SplitOperand ac = a, bc = b;
    ac.X = a.X + b0 * a.xstride;
    bc.X = b.X + b0 * b.xstride;
    ac.out = a.out + b0 * P * a.R * Kp;
    bc.out = b.out + b0 * P * b.R * Kp;
    dim3 grid(unsigned(Kp / 64), unsigned(rt), unsigned(2 * nb));
    split_bf16_kernel<P><<<grid, 256, 0, h->stream>>>(ac, bc, K, Kp);
    GB_TRY(after_launch("split_bf16"));
  }
  return GBBLAS_STATUS_SUCCESS;
}

template <int BN, int P, int STAGES, bool PARTIAL>
static gbblas_status_t launch_tc(gbblas_handle_t h, const CUtensorMap& ta, const CUtensorMap& tb, int64_t M,
                                 int64_t N, int64_t nk, int64_t batch, int split, float alpha, float beta, float* C,
                                 int64_t ldc, int64_t stride_c, float* ws, int raster_m) {
  using Cfg = TcCfg<BN, P, STAGES>;
  static std::atomic<uint64_t> attr{0};
  GB_CUDA_TRY(raise_smem_limit(attr, reinterpret_cast<const void*>(gemm_split_bf16_kernel<BN, P, STAGES, PARTIAL>),
                               Cfg::SMEM, h->device));
  const int kb_per = int(cdiv(nk, split));
  const unsigned tn = unsigned(cdiv(N, BN)), tm = unsigned(cdiv(M, kTcBM));
  dim3 grid(raster_m == 1 ? tm : tn, raster_m == 1 ? tn : tm, unsigned(batch * split));
  if (grid.y > 65535) return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: grid too large");
  // launched early (PDL): its CTAs set up while the split pass drains
  const cudaError_t le = launch_pdl(true, gemm_split_bf16_kernel<BN, P, STAGES, PARTIAL>, grid, dim3(kTcThreads),
                                    size_t(Cfg::SMEM), h->stream, ta, tb, int(M), int(N), int(nk), split, kb_per,
                                    alpha, beta, C, ldc, stride_c, ws, raster_m, h->dev_error);
  if (le != cudaSuccess) return cuda_fail(le, "gemm_split_bf16");
  return after_launch("gemm_split_bf16");
}

// 256 x 128 tiles on CTA pairs (x3 only, no split-K): a persistent grid of
// the clusters that can be resident at once (two CTAs each).
static gbblas_status_t launch_tc_pair(gbblas_handle_t h, const CUtensorMap& ta, const CUtensorMap& tb, int64_t M,
                                      int64_t N, int64_t nk, int64_t batch, float alpha, float beta, float* C,
                                      int64_t ldc, int64_t stride_c) {
  constexpr int STAGES = 4;
  using Cfg = PairCfg<STAGES>;
  auto* kern = gemm_split_bf16_pair_kernel<STAGES>;
  static std::atomic<uint64_t> attr{0};
  GB_CUDA_TRY(raise_smem_limit(attr, reinterpret_cast<const void*>(kern), Cfg::SMEM, h->device));
  const int64_t tiles = cdiv(M, 2 * kTcBM) * cdiv(N, kPairBN) * batch;
  if (tiles > INT32_MAX / 2) return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: too many tiles");
  // resident clusters, asked once per device (the static schedule assumes
  // every cluster of the grid runs at the same time)
  static std::atomic<int> resident[64];
  int clusters = (h->device >= 0 && h->device < 64) ? resident[h->device].load(std::memory_order_acquire) : 0;
  if (clusters <= 0) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * unsigned(h->sm_count / 2), 1, 1);
    cfg.blockDim = dim3(kPairThreads, 1, 1);
    cfg.dynamicSmemBytes = Cfg::SMEM;
    cfg.stream = h->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    GB_CUDA_TRY(cudaOccupancyMaxActiveClusters(&clusters, reinterpret_cast<const void*>(kern), &cfg));
    if (clusters < 1) return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: no CTA pair can be resident");
    if (h->device >= 0 && h->device < 64) resident[h->device].store(clusters, std::memory_order_release);
  }
  const int64_t grid_clusters = std::min<int64_t>(tiles, clusters);
  // placed early (programmatic dependent launch) while the split pass
  // drains; the grid is the resident clusters, so it cannot land unevenly
  const cudaError_t le = launch_pdl(true, kern, dim3(unsigned(2 * grid_clusters)), dim3(kPairThreads), Cfg::SMEM,
                                    h->stream, ta, tb, int(M), int(N), int(nk), int(tiles), alpha, beta, C, ldc,
                                    stride_c, h->dev_error);
  if (le != cudaSuccess) return cuda_fail(le, "gemm_split_bf16_pair");
  return after_launch("gemm_split_bf16_pair");
}

// 256 x 256 tiles on CTA pairs (x3: three 64 KB stages; x6: two 96 KB
// stages; no split-K): a persistent grid of the clusters that can be
// resident at once.
template <int P>
static gbblas_status_t launch_tc_pair256(gbblas_handle_t h, const CUtensorMap& ta, const CUtensorMap& tb,
                                         const CUtensorMap& tb_half, int64_t M, int64_t N, int64_t nk,
                                         int64_t batch, float alpha, float beta, float* C, int64_t ldc,
                                         int64_t stride_c) {
  constexpr int STAGES = P == 2 ? 3 : 2;
  using Cfg = Pair2Cfg<P, STAGES>;
  auto* kern = gemm_split_bf16_pair256_kernel<P, STAGES>;
  static std::atomic<uint64_t> attr{0};
  GB_CUDA_TRY(raise_smem_limit(attr, reinterpret_cast<const void*>(kern), Cfg::SMEM, h->device));
  const int64_t tiles = cdiv(M, 2 * kTcBM) * cdiv(N, kPair2BN) * batch;
  if (tiles > INT32_MAX / 2) return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: too many tiles");
  static std::atomic<int> resident[64];
  int clusters = (h->device >= 0 && h->device < 64) ? resident[h->device].load(std::memory_order_acquire) : 0;
  if (clusters <= 0) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * unsigned(h->sm_count / 2), 1, 1);
    cfg.blockDim = dim3(kPair2Threads, 1, 1);
    cfg.dynamicSmemBytes = Cfg::SMEM;
    cfg.stream = h->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    GB_CUDA_TRY(cudaOccupancyMaxActiveClusters(&clusters, reinterpret_cast<const void*>(kern), &cfg));
    if (clusters < 1) return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: no CTA pair can be resident");
    if (h->device >= 0 && h->device < 64) resident[h->device].store(clusters, std::memory_order_release);
  }
  // a last round of at most half the clusters runs as 256 x 128 halves
  // (one per cluster): 8192^3 has 13 rounds of 76 tiles and 36 more
  int64_t whole = tiles, items = tiles;
  const int64_t leftover = tiles % clusters;
  if (tiles > clusters && leftover > 0 && 2 * leftover <= clusters) {
    whole = tiles - leftover;
    items = whole + 2 * leftover;
  }
  const int64_t grid_clusters = std::min<int64_t>(items, clusters);
  const cudaError_t le = launch_pdl(true, kern, dim3(unsigned(2 * grid_clusters)), dim3(kPair2Threads), Cfg::SMEM,
                                    h->stream, ta, tb, tb_half, int(M), int(N), int(nk), int(whole), int(items),
                                    alpha, beta, C, ldc, stride_c, h->dev_error);
  if (le != cudaSuccess) return cuda_fail(le, "gemm_split_bf16_pair256");
  return after_launch("gemm_split_bf16_pair256");
}

template <int BN, int P>
static gbblas_status_t split_gemm_run(gbblas_handle_t h, const GemmArgs<float>& g, int split, int raster_m,
                                      int pair = 0) {
  constexpr int STAGES = (P * (kTcBM + BN) * kTcBK * 2) <= 56 * 1024 ? 4 : ((P * (kTcBM + BN) * kTcBK * 2) <= 72 * 1024 ? 3 : 2);
  const int64_t M = g.m, N = g.n, K = g.k, B = g.batch;
  const int64_t Kp = cdiv(K, kTcBK) * kTcBK;
  const int64_t nk = Kp / kTcBK;
  if (split < 1) split = 1;
  if (split > nk) split = int(nk);
  split = int(cdiv(nk, cdiv(nk, split)));  // no empty slices
  if (B * split > 65535) return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: batch x split too large");
  if (split > 1 && double(split) * double(M) * double(N) * double(B) > double(int64_t(1) << 28))
    return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: split-K workspace too large");
  const size_t a_bytes = (size_t(P) * M * Kp * 2 * B + 1023) & ~size_t(1023);
  const size_t b_bytes = (size_t(P) * N * Kp * 2 * B + 1023) & ~size_t(1023);
  const size_t w_bytes = split > 1 ? sizeof(float) * size_t(split) * M * N * B : 0;
  void* wsp = nullptr;
  GB_TRY(temp_acquire(h, a_bytes + b_bytes + w_bytes, &wsp));
  auto* at = static_cast<__nv_bfloat16*>(wsp);
  auto* bt = reinterpret_cast<__nv_bfloat16*>(static_cast<uint8_t*>(wsp) + a_bytes);
  float* ws = split > 1 ? reinterpret_cast<float*>(static_cast<uint8_t*>(wsp) + a_bytes + b_bytes) : nullptr;
  // A(m, k): (ta ? A[k + m*lda] : A[m + k*lda]);  B as rows n: (tb ? B[n + k*ldb] : B[k + n*ldb])
  GB_TRY(launch_split<P>(h, split_operand(g.a, g.ta ? g.lda : 1, g.ta ? 1 : g.lda, M, g.stride_a, at),
                         split_operand(g.b, g.tb ? 1 : g.ldb, g.tb ? g.ldb : 1, N, g.stride_b, bt), K, Kp, B));
  CUtensorMap ma, mb;
  GB_TRY(make_term_map(&ma, at, M, Kp, P * B, kTcBM));
  if (pair == 1 && P == 2 && split == 1) {
    GB_TRY(make_term_map(&mb, bt, N, Kp, P * B, kPairBHalf));
    return launch_tc_pair(h, ma, mb, M, N, nk, B, g.alpha, g.beta, g.c, g.ldc, g.stride_c);
  }
  if (pair == 2 && split == 1) {
    CUtensorMap mbh;  // B rows of a 256 x 128 half item (64 per CTA)
    GB_TRY(make_term_map(&mb, bt, N, Kp, P * B, kPair2BHalf));
    GB_TRY(make_term_map(&mbh, bt, N, Kp, P * B, kPair2BHalf / 2));
    return launch_tc_pair256<P>(h, ma, mb, mbh, M, N, nk, B, g.alpha, g.beta, g.c, g.ldc, g.stride_c);
  }
  GB_TRY(make_term_map(&mb, bt, N, Kp, P * B, BN));
  if (split == 1)
    return launch_tc<BN, P, STAGES, false>(h, ma, mb, M, N, nk, B, 1, g.alpha, g.beta, g.c, g.ldc, g.stride_c,
                                           nullptr, raster_m);
  GB_TRY((launch_tc<BN, P, STAGES, true>(h, ma, mb, M, N, nk, B, split, g.alpha, g.beta, g.c, g.ldc, g.stride_c,
                                         ws, raster_m)));
  return launch_splitk_reduce(h, g, split, ws);
}

gbblas_status_t launch_gemm_split_bf16_cfg(gbblas_handle_t h, const GemmArgs<float>& g, int pieces, int bn,
                                           int split, int raster_m) {
  if (pieces != 2 && pieces != 3) return fail(GBBLAS_STATUS_INVALID_ARG, "split-BF16 GEMM: pieces must be 2 or 3");
  if (g.m > INT32_MAX / 2 || g.n > INT32_MAX / 2 || g.k > INT32_MAX / 2)
    return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: dimension too large");
  if (g.k == 0) return launch_scale_c(h, g.m, g.n, g.beta, g.c, g.ldc, g.stride_c, g.batch);
  if (bn == 64)
    return pieces == 2 ? split_gemm_run<64, 2>(h, g, split, raster_m) : split_gemm_run<64, 3>(h, g, split, raster_m);
  if (bn == 128)
    return pieces == 2 ? split_gemm_run<128, 2>(h, g, split, raster_m)
                       : split_gemm_run<128, 3>(h, g, split, raster_m);
  return fail(GBBLAS_STATUS_INVALID_ARG, "split-BF16 GEMM: N tile must be 64 or 128");
}

// CTA-pair tiles for the x3 mode (GBBLAS_PAIR_TILES=0 turns them off).
static bool pair_tiles_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("GBBLAS_PAIR_TILES");
    return !(v && v[0] == '0');
  }();
  return on;
}

// 256 x 256 CTA-pair tiles: M and N at least 256, tiles for at least half
// of the resident clusters, and useful work per round (the rounds' fill
// times the share of each tile inside the problem) at least 0.8 x that of
// 128 x 128 one-CTA tiles (the pair tile's MMA rate per SM is about 1.3 x
// higher); a short last round run as 256 x 128 halves counts 0.6 of a
// round.  x3 / x6 TFLOP/s against the next choice: 2048^3 267 / 185 against
// 225 / 170, 2560^3 325 / 199 against 292 / 183, 3072^3 430 / 250 against
// 358 / 208, 6144^3 572 / 308 against 452 / 252; strided batches of 384^3
// and 300^3 (tiles a quarter to two thirds padding) ran 7-9% slower on the
// pair tiles, and the rule leaves them out.
bool split_bf16_pair256_fits(const GemmArgs<float>& g, int64_t sm) {
  if (g.k <= 0 || g.m < 2 * kTcBM || g.n < kPair2BN || !pair_tiles_enabled()) return false;
  const int64_t clusters = sm / 2;
  const int64_t m256 = cdiv(g.m, 2 * kTcBM), n256 = cdiv(g.n, kPair2BN);
  const int64_t m128 = cdiv(g.m, kTcBM), n128 = cdiv(g.n, 128);
  const int64_t t256 = m256 * n256 * g.batch, t128 = m128 * n128 * g.batch;
  if (clusters < 1 || 2 * t256 < clusters) return false;
  const double mn = double(g.m) * double(g.n);
  const double use256 = mn / (double(m256 * 2 * kTcBM) * double(n256 * kPair2BN));
  const double use128 = mn / (double(m128 * kTcBM) * double(n128 * 128));
  // a last round of at most half the clusters runs as 256 x 128 halves,
  // about 0.6 of a round
  const int64_t left = t256 % clusters, whole_rounds = t256 / clusters;
  const double rounds = double(whole_rounds) +
                        (left == 0 ? 0.0 : (whole_rounds > 0 && 2 * left <= clusters ? 0.6 : 1.0));
  const double fill256 = double(t256) / (rounds * double(clusters));
  const double fill128 = double(t128) / double(cdiv(t128, sm) * sm);
  return fill256 * use256 >= 0.8 * fill128 * use128;
}

// The fixed split-BF16 modes: 256 x 256 CTA-pair tiles (x3 and x6) where
// split_bf16_pair256_fits; else 256 x 128 CTA-pair tiles (x3) when there are
// at least two waves of 128 x 128 tiles; 128 x 128 tiles when they fill the
// SMs; else 128 x 64 tiles; and when even those leave half the SMs idle,
// split-K slices of at least 4 k-blocks.
SplitBf16Route split_bf16_route(const GemmArgs<float>& g, int pieces, int64_t sm) {
  if (split_bf16_pair256_fits(g, sm)) return {2 * kTcBM, kPair2BN, 1};
  const int64_t tm = cdiv(g.m, kTcBM);
  const int64_t t128 = tm * cdiv(g.n, 128) * g.batch;
  if (pieces == 2 && t128 >= 2 * sm && g.k > 0 && pair_tiles_enabled()) return {2 * kTcBM, 128, 1};
  if (t128 >= sm || g.n <= 64) return {kTcBM, 128, 1};
  const int64_t t64 = tm * cdiv(g.n, 64) * g.batch;
  int64_t split = 1;
  if (2 * t64 <= sm) {
    split = sm / t64;
    const int64_t deep = cdiv(g.k, kTcBK) / 4;
    if (split > deep) split = deep;
    if (split > 16) split = 16;
    if (split < 1) split = 1;
  }
  return {kTcBM, 64, int(split)};
}

gbblas_status_t launch_gemm_split_bf16(gbblas_handle_t h, const GemmArgs<float>& g, int pieces) {
  // the kernels take M, N and the k-block count as int (the CTA-pair paths
  // included)
  if (g.m > INT32_MAX / 2 || g.n > INT32_MAX / 2 || g.k > INT32_MAX / 2)
    return fail(GBBLAS_STATUS_UNSUPPORTED, "split-BF16 GEMM: dimension too large");
  const SplitBf16Route r = split_bf16_route(g, pieces, h->sm_count);
  if (r.tile_m == 2 * kTcBM) {
    if (r.tile_n == kPair2BN)
      return pieces == 2 ? split_gemm_run<128, 2>(h, g, 1, 0, 2) : split_gemm_run<128, 3>(h, g, 1, 0, 2);
    return split_gemm_run<128, 2>(h, g, 1, 0, 1);
  }
  return launch_gemm_split_bf16_cfg(h, g, pieces, r.tile_n, r.k_slices, r.tile_n == 128 ? 2 : 0);
}

}  // namespace gb

using namespace gb;

extern "C" {

gbblas_status_t gbblas_sgemm_split_route(int64_t m, int64_t n, int64_t k, int64_t batch, int mode, int sm_count,
                                         int* tile_m, int* tile_n, int* k_slices) {
  clear_error();
  if (m < 0 || n < 0 || k < 0 || batch < 0)
    return fail(GBBLAS_STATUS_INVALID_ARG, "sgemm_split_route: negative dimension");
  if (mode != GBBLAS_SGEMM_SPLIT_BF16X3 && mode != GBBLAS_SGEMM_SPLIT_BF16X6)
    return fail(GBBLAS_STATUS_INVALID_ARG, "sgemm_split_route: mode must be SPLIT_BF16X3 or SPLIT_BF16X6");
  if (sm_count < 1) return fail(GBBLAS_STATUS_INVALID_ARG, "sgemm_split_route: sm_count must be positive");
  if (m > INT32_MAX / 2 || n > INT32_MAX / 2 || k > INT32_MAX / 2)
    return fail(GBBLAS_STATUS_UNSUPPORTED, "sgemm_split_route: dimension too large");
  GemmArgs<float> g{};
  g.m = m;
  g.n = n;
  g.k = k;
  g.batch = batch;
  const SplitBf16Route r = split_bf16_route(g, mode == GBBLAS_SGEMM_SPLIT_BF16X3 ? 2 : 3, sm_count);
  if (tile_m) *tile_m = r.tile_m;
  if (tile_n) *tile_n = r.tile_n;
  if (k_slices) *k_slices = r.k_slices;
  return GBBLAS_STATUS_SUCCESS;
}

}  // extern "C"

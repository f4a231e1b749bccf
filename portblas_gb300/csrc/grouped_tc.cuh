// grouped_tc.cuh — tensor-core (tcgen05) path of the grouped GEMM.
//
// Two kernels, captured together in the plan's CUDA graph:
//
// 1. grouped_split_kernel<T, P>: converts every operand that needs it into
//    K-major BF16 terms [P][rows][Kp] (Kp = k rounded up to 16, zero pad):
//    K-contiguous operands in 32-row x 128-k tiles, the others transposed
//    through 64 x 64 shared-memory tiles, so both the strided read and the
//    K-contiguous write are coalesced.  FP32 inputs are
//    split into P = 3 terms with exact residuals (as in gemm_tc.cu), so the
//    six kept term products give FP32-level accuracy at any k; BF16 inputs
//    are one term, and a BF16 operand that is already K-contiguous with a
//    16-byte-aligned leading dimension is read in place (no conversion).
//    Each element is converted once, however many output tiles read it.
//
// 2. grouped_tc_kernel<P>: persistent CTAs over the 128 x 128 output tiles of
//    all problems (problems ordered by decreasing K per tile, tiles numbered
//    in that order, a global atomic counter hands them out; a long-K problem
//    may have its K cut into slices, see the split-K note below).  Every operand has its
//    own TMA tensor map (in device memory, two per problem), so the operand
//    tiles stream in with cp.async.bulk.tensor exactly as in the dense
//    kernel, and the pipeline never drains at a tile boundary:
//      warp 2     scheduler: takes tile numbers from the counter, resolves
//                 their problems and fills a ring of work slots ahead of the
//                 other roles (and prefetches the tiles' tensor maps);
//      warp 0     producer: issues the TMA loads of each slot's k-blocks into
//                 an S-stage mbarrier ring (the P terms of A and of B in one
//                 3-D box each);
//      warp 1     allocates TMEM; one lane issues tcgen05.mma (M128 K16;
//                 N128 for every term pair of one or two terms, and for three
//                 terms the six products as four MMAs, two of them N256 over
//                 adjacent B terms), commits each stage back to the producer
//                 and each finished chunk of CHUNK k-blocks to one of the
//                 TMEM accumulators (four of 128 columns for BF16 inputs, two
//                 of 256 for FP32);
//      warps 3-10 epilogue: tcgen05.ld of each chunk into FP32 registers
//                 (64 columns of one output row per thread), then
//                 alpha / beta and the stores to C (or, for a K slice, the
//                 partial block and the slice fold), while the MMA warp is
//                 already filling the other accumulator.
// Every mbarrier wait is bounded: a wait that gives up records an error code
// and its role stops; the others give up on their own bounded waits, the
// producer waits for its copies in flight, and TMEM is freed.
#pragma once

#include <cuda_bf16.h>

#include "tc_ptx.cuh"

namespace gb {

// Warps: 0 producer, 1 MMA issuer, 2 scheduler, 3..10 epilogue.
constexpr int kGtBM = 128, kGtBN = 128, kGtBK = 64, kGtEpiWarps = 8, kGtThreads = 32 * (3 + kGtEpiWarps),
              kGtRing = 8, kGtGroupM = 8;
// K depth of one TMEM chunk before its promotion into FP32 registers (a
// shallower chunk keeps more of the sum in FP32; 128 costs no time here)
constexpr int kGtChunkK = 128;

template <int P>
struct GtCfg {
  // k per stage: 64 (128-byte swizzled rows) for one or two terms, 32
  // (64-byte swizzle) for three, so four stages fit and three are in flight
  static constexpr int BK = P == 3 ? 32 : kGtBK;
  static constexpr int A_TILE = kGtBM * BK * 2;  // per term
  static constexpr int B_TILE = kGtBN * BK * 2;
  static constexpr int STAGE = P * (A_TILE + B_TILE);
  static constexpr int STAGES = P == 1 ? 6 : (P == 2 ? 3 : 4);
  // TMEM chunk accumulators (the MMA warp runs up to NACC - 1 chunks ahead
  // of the epilogue): four of 128 columns for one or two terms, two of 256
  // for three
  static constexpr int NACC = P == 3 ? 2 : 4;
  // barriers: full/empty per stage, two accumulator pairs, a work-slot pair per ring entry; then the TMEM address
  static constexpr int BARRIER_BYTES = (2 * STAGES + 2 * NACC + 2 * kGtRing) * 8 + 4;
  static constexpr int SMEM = STAGES * STAGE + 1024 + 512;
  static constexpr int NPAIRS = P == 1 ? 1 : 3;  // term products issued one by one (P <= 2)
  // columns of one chunk accumulator: with P = 3 the products of an A term
  // with the two adjacent leading B terms are one N = 256 MMA, and the
  // epilogue adds the two column halves
  static constexpr int ACC = P == 3 ? 2 * kGtBN : kGtBN;
  static constexpr int TMEM_COLS = NACC * ACC;  // the chunk accumulators
  static_assert(TMEM_COLS <= 512, "tensor memory budget");
  static_assert(BARRIER_BYTES <= 512, "barrier area");
  static_assert(SMEM <= 227 * 1024, "shared memory budget");
};

// One operand to convert: X(r, k) = src[r*sr + k*sk], r < rows, k < K,
// written for k < Kp (zeros for k >= K): BF16 as out[r][k] (Kp a multiple of
// 16, so every row starts on a 32-byte sector), FP32's three terms
// k-block-major as out[k / 32][p][r][k % 32] (Kp a multiple of 32;
// gt_term3_ptr).
struct GtOperand {
  const void* src;
  int64_t sr, sk;
  int rows, K, Kp, blocks;  // blocks: tiles of the mapping gt_split_blocks() picks
  int parts;                // CTAs sharing the operand's tiles
  __nv_bfloat16* out;
};

// tiles each CTA of the split pass converts (an operand of b tiles gets
// ceil(b / kGtSplitTiles) CTAs, so every CTA has about the same work)
constexpr int kGtSplitTiles = 2;

// Tiles of an operand's conversion: K-contiguous operands (sk == 1) with no
// transpose, BF16 ones (flat) in blocks of kGtFlat consecutive elements of
// the rows x Kp output (short rows share a block), FP32 ones (three terms)
// in 32-row x 128-k tiles; the others in 64 x 64 tiles transposed through
// shared memory.
constexpr int kGtFlat = 4096;
__host__ __device__ inline int64_t gt_split_blocks(int64_t rows, int64_t Kp, bool kcontig, bool flat) {
  if (!kcontig) return ((rows + 63) / 64) * ((Kp + 63) / 64);
  return flat ? (rows * Kp + kGtFlat - 1) / kGtFlat : ((rows + 31) / 32) * ((Kp + 127) / 128);
}

// Element (term p, row r, k) of an FP32 operand's three BF16 terms, stored
// k-block-major as [Kp / 32][3][rows][32] (Kp a multiple of 32): the tile
// kernel's box for one 32-deep k-block (32 k x 128 rows x 3 terms) is then
// one contiguous run instead of 384 separate 64-byte row pieces.
__device__ __forceinline__ __nv_bfloat16* gt_term3_ptr(__nv_bfloat16* out, int64_t rows, int64_t r, int64_t k,
                                                       int p) {
  return out + (((k >> 5) * 3 + p) * rows + r) * 32 + (k & 31);
}

template <typename T>
__device__ __forceinline__ float gt_ld(const T* p);
template <>
__device__ __forceinline__ float gt_ld<float>(const float* p) { return __ldg(p); }
template <>
__device__ __forceinline__ float gt_ld<__nv_bfloat16>(const __nv_bfloat16* p) {
  return __uint_as_float(uint32_t(__ldg(reinterpret_cast<const unsigned short*>(p))) << 16);
}

// Four consecutive values of one row at p (k .. k+3, those >= kend read as 0).
template <typename T>
__device__ __forceinline__ void gt_ld4(const T* p, int64_t k, int64_t kend, float (&v)[4]) {
  if (k + 3 < kend) {
    if (sizeof(T) == 4 && (reinterpret_cast<uintptr_t>(p) & 15) == 0) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(p));
      v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
      return;
    }
    if (sizeof(T) == 2 && (reinterpret_cast<uintptr_t>(p) & 7) == 0) {
      const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
      v[0] = __uint_as_float(q.x << 16); v[1] = __uint_as_float(q.x & 0xffff0000u);
      v[2] = __uint_as_float(q.y << 16); v[3] = __uint_as_float(q.y & 0xffff0000u);
      return;
    }
  }
#pragma unroll
  for (int e = 0; e < 4; ++e) v[e] = k + e < kend ? gt_ld<T>(p + e) : 0.f;
}

// Four consecutive raw BF16 values of one row at p (k .. k+3, those >= kend
// read as 0), packed two per word; no byte outside the four values is read.
__device__ __forceinline__ uint2 gt_ld4_raw(const __nv_bfloat16* p, int64_t k, int64_t kend) {
  const unsigned short* h = reinterpret_cast<const unsigned short*>(p);
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  if (k + 3 < kend) {
    if ((a & 7) == 0) return __ldg(reinterpret_cast<const uint2*>(p));
    if ((a & 3) == 0) {
      const unsigned int* w = reinterpret_cast<const unsigned int*>(p);
      return make_uint2(__ldg(w), __ldg(w + 1));
    }
    const uint32_t mid = __ldg(reinterpret_cast<const unsigned int*>(a + 2));
    return make_uint2(uint32_t(__ldg(h)) | (mid << 16), (mid >> 16) | (uint32_t(__ldg(h + 3)) << 16));
  }
  uint32_t e[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) e[i] = k + i < kend ? uint32_t(__ldg(h + i)) : 0u;
  return make_uint2(e[0] | (e[1] << 16), e[2] | (e[3] << 16));
}

// P BF16 terms of n consecutive FP32 values, t_0 = bf16(x), t_{i+1} =
// bf16(x - t_0 - ... - t_i) (exact residuals), packed two per word; term p of
// pair e goes to w[p][e].
template <int P, int NPAIR>
__device__ __forceinline__ void gt_terms(float* x, uint32_t (&w)[P][NPAIR]) {
#pragma unroll
  for (int p = 0; p < P; ++p)
#pragma unroll
    for (int e = 0; e < NPAIR; ++e) {
      const __nv_bfloat162 h2 = __floats2bfloat162_rn(x[2 * e], x[2 * e + 1]);
      w[p][e] = *reinterpret_cast<const uint32_t*>(&h2);
      if (p + 1 < P) {
        x[2 * e] -= __uint_as_float(w[p][e] << 16);
        x[2 * e + 1] -= __uint_as_float(w[p][e] & 0xffff0000u);
      }
    }
}

// CTA b converts tiles y, y + parts, ... of operand o, (o, y) = ctas[b]; the
// CTAs of one operand are consecutive and the largest operands come first.
// Every
// thread has 16 global loads in flight per tile and writes whole 32-byte
// sectors of the term rows.
template <typename T, int P>
__global__ void __launch_bounds__(256, 8) grouped_split_kernel(const GtOperand* __restrict__ ops,
                                                               const int2* __restrict__ ctas) {
  __shared__ float tile[64][65];  // transposing mapping: tile[k][r]
  const int2 cta = ctas[blockIdx.x];
  const GtOperand op = ops[cta.x];
  const int part = cta.y;
  const T* __restrict__ X = static_cast<const T*>(op.src);
  __nv_bfloat16* __restrict__ out = op.out;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if constexpr (sizeof(T) == 2) {
    if (op.sk == 1) {
      // K-contiguous BF16 (its own single term: the raw 16-bit values move):
      // block j is elements [j * kGtFlat, +kGtFlat) of the rows x Kp output,
      // row after row; lane l of warp w moves the four elements from
      // w * kGtFlat / 8 + 128 i + 4 l (i < 4): rows shorter than 128 pack into
      // one warp step instead of leaving lanes idle (Kp is a multiple of 16,
      // so a 4-element group never crosses a row)
      const int64_t total = int64_t(op.rows) * op.Kp;
      const int rq = 128 / op.Kp, rk = 128 % op.Kp;  // a 128-element step in rows and columns
      const __nv_bfloat16* Xh = reinterpret_cast<const __nv_bfloat16*>(X);
      for (int j = part; j < op.blocks; j += op.parts) {
        const int64_t e0 = int64_t(j) * kGtFlat + warp * (kGtFlat / 8) + 4 * lane;
        if (e0 >= total) continue;
        int64_t rr[4];
        int kk[4];
        rr[0] = e0 / op.Kp;
        kk[0] = int(e0 - rr[0] * op.Kp);
#pragma unroll
        for (int i = 1; i < 4; ++i) {
          kk[i] = kk[i - 1] + rk;
          rr[i] = rr[i - 1] + rq;
          if (kk[i] >= op.Kp) {
            kk[i] -= op.Kp;
            ++rr[i];
          }
        }
        uint2 q[4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
          q[i] = rr[i] < op.rows ? gt_ld4_raw(Xh + rr[i] * op.sr + kk[i], kk[i], op.K) : make_uint2(0u, 0u);
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (rr[i] < op.rows) *reinterpret_cast<uint2*>(out + rr[i] * op.Kp + kk[i]) = q[i];
      }
      return;
    }
  }
  if (op.sk == 1) {
    // K-contiguous FP32: warp w converts rows 4w .. 4w+3 of a 32 x 128 tile,
    // lane l the four k from 4l
    const int nkb = (op.Kp + 127) / 128;
    for (int j = part; j < op.blocks; j += op.parts) {
      const int64_t r0 = int64_t(j / nkb) * 32 + warp * 4, k = int64_t(j % nkb) * 128 + 4 * lane;
      float v[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t r = r0 + i;
        if (r < op.rows) {
          gt_ld4<T>(X + r * op.sr + k, k, op.K, v[i]);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) v[i][e] = 0.f;
        }
      }
      if (k < op.Kp) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int64_t r = r0 + i;
          if (r < op.rows) {
            uint32_t w[P][2];
            gt_terms<P, 2>(v[i], w);
#pragma unroll
            for (int p = 0; p < P; ++p)
              *reinterpret_cast<uint2*>(gt_term3_ptr(out, op.rows, r, k, p)) = make_uint2(w[p][0], w[p][1]);
          }
        }
      }
    }
    return;
  }
  // rows contiguous (sr == 1): 64 x 64 tiles through shared memory; loads
  // with lanes along r, then each thread writes 16-byte chunks (8 k) of two rows
  const int nkb = (op.Kp + 63) / 64;
  for (int j = part; j < op.blocks; j += op.parts) {
    const int64_t r0 = int64_t(j / nkb) * 64, k0 = int64_t(j % nkb) * 64;
    if constexpr (sizeof(T) == 2) {
      // BF16: transpose the raw 16-bit values (64 rows of 130 halfwords)
      unsigned short(*th)[130] = reinterpret_cast<unsigned short(*)[130]>(&tile[0][0]);
      const unsigned short* Xh = reinterpret_cast<const unsigned short*>(X);
      const int rr = t & 63;
      const bool row_ok = r0 + rr < op.rows;
      // column k0 + kk of this thread's row; the next column is 4 * sk on
      const int kq = (t >> 6);
      const unsigned short* q = Xh + (row_ok ? r0 + rr : 0) + (k0 + kq) * op.sk;
      const int64_t step = 4 * op.sk;
      const int64_t kleft = op.K - k0 - kq;  // columns of this thread still inside K, from i = 0
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        th[kq + 4 * i][rr] = (row_ok && 4 * i < kleft) ? __ldg(q + i * step) : (unsigned short)0;
      }
      __syncthreads();
      const int c = t & 7;
      const int64_t k = k0 + 8 * c;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int rq = (t >> 3) + 32 * h;
        if (r0 + rq < op.rows && k < op.Kp) {
          uint32_t w[4];
#pragma unroll
          for (int e = 0; e < 4; ++e)
            w[e] = uint32_t(th[8 * c + 2 * e][rq]) | (uint32_t(th[8 * c + 2 * e + 1][rq]) << 16);
          *reinterpret_cast<uint4*>(out + (r0 + rq) * op.Kp + k) = make_uint4(w[0], w[1], w[2], w[3]);
        }
      }
      __syncthreads();
      continue;
    }
    {
      const int rr = t & 63;
      const bool row_ok = r0 + rr < op.rows;
      const int kq = (t >> 6);
      const T* q = X + (row_ok ? r0 + rr : 0) + (k0 + kq) * op.sk;
      const int64_t step = 4 * op.sk;
      const int64_t kleft = op.K - k0 - kq;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        tile[kq + 4 * i][rr] = (row_ok && 4 * i < kleft) ? gt_ld<T>(q + i * step) : 0.f;
      }
    }
    __syncthreads();
    const int c = t & 7;
    const int64_t k = k0 + 8 * c;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int rr = (t >> 3) + 32 * h;
      const int64_t r = r0 + rr;
      if (r < op.rows && k < op.Kp) {
        float x[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) x[e] = tile[8 * c + e][rr];
        uint32_t w[P][4];
        gt_terms<P, 4>(x, w);
#pragma unroll
        for (int p = 0; p < P; ++p)
          *reinterpret_cast<uint4*>(gt_term3_ptr(out, op.rows, r, k, p)) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
      }
    }
    __syncthreads();
  }
}

// Split-K: a problem whose tiles are much longer (in K) than the average work
// per SM is cut into `splits` K slices per output tile; its tiles are
// numbered slice-major (tile = slice * output tiles + output tile).  Each
// epilogue warp owns a 32-row x 64-column sub-block of the output tile (a
// sub-block wholly outside the problem is skipped); it writes its slice's
// FP32 partial sub-block (column-major, 32 lanes per column, so the stores
// coalesce) and the partials are folded up a tree of fan-in kGtFoldFan:
// slices 8i .. 8i+7 form node i of level 1, nodes 8j .. 8j+7 of level 1 form
// node j of level 2, and so on up to one root.  Every node has a ticket per
// sub-block; the child warp that takes a node's last ticket adds the node's
// children in index order (so the sum does not depend on the arrival
// order), resets the ticket (a graph can replay the launch) and, below the
// root, stores the node's partial in its first child's slot and climbs;
// the warp that completes the root applies alpha / beta and stores C.  Only
// the last slice to finish waits for a level's reads, so the fold adds about
// kGtFoldFan reads per level to the tile instead of one per slice.  No
// barrier spans warps.
constexpr int kGtSubs = 8;                  // epilogue sub-blocks per output tile
constexpr int kGtSubFloats = 32 * 64;       // floats per sub-block
constexpr int kGtTileFloats = kGtSubs * kGtSubFloats;
constexpr int kGtFoldFan = 8;

// Internal nodes of the fold tree of `splits` slices (tickets per sub-block).
__host__ __device__ inline int gt_fold_nodes(int splits) {
  int t = 0;
  for (int n = splits; n > 1;) {
    n = (n + kGtFoldFan - 1) / kGtFoldFan;
    t += n;
  }
  return t;
}

// One scheduled tile (prob < 0: no more tiles).
struct GtWork {
  int prob, nk, m0, n0;  // problem, k-blocks of this slice, tile origin
  int mn;                // bit 0 / 1: A / B tiles are MN-major (rows contiguous, read in place)
  int m, n;              // the problem's C extent
  int kb0;               // first k-block of this slice
  int slice, splits;     // K slice of the output tile, and their number
  float alpha, beta;
  float* c;
  int64_t ldc;
  float* part;           // split-K: slice 0's partial block of this output tile
  unsigned int* tick;    // split-K: the output tile's tickets, [fold node][kGtSubs]
};

// tiles the scheduler takes from the counter at a time
constexpr int kGtBatch = 8;

// MN-major BF16 tiles (operands read in place with their rows contiguous):
// two TMA boxes of kGtMnBox rows (128 bytes) x 64 k, kGtMnAtom bytes apart;
// the descriptor's leading-dimension offset is the step between those
// 64-row atoms along MN, its stride offset the step between 8-row groups
// along K (checked against the oracle: the swapped assignment gives wrong
// products, not a fault, since both stay inside the stage)
constexpr int kGtMnBox = 64, kGtMnAtom = kGtMnBox * kGtBK * 2;
constexpr uint32_t kGtMnLbo = kGtMnAtom, kGtMnSbo = 1024;

enum : int { kErrGtProducer = 401, kErrGtMma = 402, kErrGtEpilogue = 403, kErrGtDrain = 404 };

__device__ __forceinline__ void tensormap_acquire(const CUtensorMap* map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(map))
               : "memory");
}

// probs: problem table (tiles numbered in table order; within a problem
// down groups of kGtGroupM tile rows, then along N); tile_prob[t]: problem
// of tile t; maps[2p], maps[2p+1]: tensor maps of problem p's A terms ([P][m][Kp]) and B terms
// ([P][n][Kp]), box 64 x rows x P; counters[0] = next tile, counters[1] =
// CTAs finished (the last one resets both, so a graph can replay the launch);
// parts / ticks: split-K partial blocks and tickets (problem fields
// part_off / tick_off index them).
template <int P, int CHUNK, class Prob>
__global__ void __launch_bounds__(kGtThreads, 1)
    grouped_tc_kernel(const Prob* __restrict__ probs, const int* __restrict__ tile_prob,
                      const CUtensorMap* __restrict__ maps, int64_t total_tiles,
                      unsigned long long* __restrict__ counters, float* __restrict__ parts,
                      unsigned int* __restrict__ ticks, int* __restrict__ err) {
  using Cfg = GtCfg<P>;
  constexpr int S = Cfg::STAGES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * Cfg::STAGE);
  uint64_t* empty = full + S;
  constexpr int NACC = Cfg::NACC;
  uint64_t* tfull = empty + S;         // [NACC] chunk accumulator ready
  uint64_t* tempty = tfull + NACC;     // [NACC] chunk accumulator drained
  uint64_t* wfull = tempty + NACC;     // [kGtRing] work slot published
  uint64_t* wempty = wfull + kGtRing;  // [kGtRing] work slot read by the producer, MMA warp and epilogue
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(wempty + kGtRing);
  __shared__ GtWork ring[kGtRing];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < NACC; ++b) {
      tc::mbar_init(&tfull[b], 1);
      tc::mbar_init(&tempty[b], kGtEpiWarps);  // one arrival per epilogue warp
    }
    for (int r = 0; r < kGtRing; ++r) {
      tc::mbar_init(&wfull[r], 1);
      tc::mbar_init(&wempty[r], 2 + kGtEpiWarps);  // producer + MMA warp + epilogue warps
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

  if (warp == 2) {
    // ----------------------------------------------------------- scheduler --
    // kGtBatch tiles per atomic (their lookups run in parallel on the
    // lanes) until the last two rounds of the grid, then one at a time so the
    // CTAs finish together
    __shared__ GtWork batch[kGtBatch];
    uint32_t i = 0;
    int take = 2ll * kGtBatch * gridDim.x >= total_tiles ? 1 : kGtBatch;
    bool more = true;
    while (more) {
      long long base = 0;
      if (lane == 0) base = (long long)atomicAdd(&counters[0], (unsigned long long)take);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (lane < take) {
        const long long tile = base + lane;
        GtWork w{};
        w.prob = -1;
        if (tile < total_tiles) {
          const int p = __ldg(tile_prob + tile);
          const Prob& pr = probs[p];
          int local = int(tile - pr.tile_start);
          const int tiles_m = (pr.m + kGtBM - 1) / kGtBM;
          const int nk_all = pr.k > 0 ? (pr.k + Cfg::BK - 1) / Cfg::BK : 0;
          w.prob = p;
          w.mn = pr.mn;
          w.splits = pr.splits;
          w.slice = 0;
          w.kb0 = 0;
          w.nk = nk_all;
          if (pr.splits > 1) {
            const int out_tiles = tiles_m * pr.tiles_n;
            w.slice = local / out_tiles;
            local -= w.slice * out_tiles;
            w.kb0 = w.slice * pr.kbs;
            w.nk = min(pr.kbs, nk_all - w.kb0);
            w.part = parts + pr.part_off + int64_t(local) * pr.splits * kGtTileFloats;
            w.tick = ticks + pr.tick_off + int64_t(local) * gt_fold_nodes(pr.splits) * kGtSubs;
          }
          // tiles of a problem go down kGtGroupM M tiles, then along N, so the
          // CTAs working at the same time share A and B panels in L2
          const int per_group = kGtGroupM * pr.tiles_n;
          const int first_m = (local / per_group) * kGtGroupM, in = local % per_group;
          const int gsize = min(tiles_m - first_m, kGtGroupM);
          w.m0 = (first_m + in % gsize) * kGtBM;
          w.n0 = (in / gsize) * kGtBN;
          w.m = pr.m;
          w.n = pr.n;
          w.alpha = pr.alpha;
          w.beta = pr.beta;
          w.c = pr.c;
          w.ldc = pr.ldc;
          if (w.nk > 0) {
            tc::tma_prefetch_desc(maps + 2 * p);
            tc::tma_prefetch_desc(maps + 2 * p + 1);
          }
        }
        batch[lane] = w;
      }
      __syncwarp();
      if (lane == 0) {
        for (int l = 0; l < take; ++l, ++i) {
          const int r = i % kGtRing;
          if (!tc::mbar_wait(&wempty[r], ((i / kGtRing) & 1) ^ 1)) {
            atomicExch(err, kErrGtProducer);
            more = false;
            break;
          }
          ring[r] = batch[l];
          tc::mbar_arrive(&wfull[r]);
          if (batch[l].prob < 0) {
            more = false;
            break;
          }
        }
      }
      more = __shfl_sync(0xffffffffu, more, 0);
      if (base + 2ll * kGtBatch * gridDim.x >= total_tiles) take = 1;
      __syncwarp();
    }
  } else if (warp == 0) {
    // ------------------------------------------------------------ producer --
    if (lane == 0) {
      uint32_t it = 0;
      int fenced = -1;  // problem whose tensor maps this thread last fenced
      for (uint32_t i = 0;; ++i) {
        const int r = i % kGtRing;
        if (!tc::mbar_wait(&wfull[r], (i / kGtRing) & 1)) {
          atomicExch(err, kErrGtProducer);
          break;
        }
        const GtWork w = ring[r];
        tc::mbar_arrive(&wempty[r]);
        if (w.prob < 0) break;
        if (w.nk == 0) continue;
        const CUtensorMap* ma = maps + 2 * w.prob;
        const CUtensorMap* mb = ma + 1;
        if (w.prob != fenced) {  // once per run of tiles of one problem
          tensormap_acquire(ma);
          tensormap_acquire(mb);
          fenced = w.prob;
        }
        bool ok = true;
        for (int kb = 0; kb < w.nk; ++kb, ++it) {
          const int s = it % S;
          if (!tc::mbar_wait(&empty[s], ((it / S) & 1) ^ 1)) {
            atomicExch(err, kErrGtProducer);
            ok = false;
            break;
          }
          tc::mbar_arrive_expect_tx(&full[s], Cfg::STAGE);
          uint8_t* st = smem + s * Cfg::STAGE;
          const int kc = (w.kb0 + kb) * Cfg::BK;
          if (P == 3) {  // k-block-major terms: plane (k-block, term)
            tc::tma_load_3d(st, ma, &full[s], 0, w.m0, (w.kb0 + kb) * P);
            tc::tma_load_3d(st + P * Cfg::A_TILE, mb, &full[s], 0, w.n0, (w.kb0 + kb) * P);
          } else {
            if (w.mn & 1) {  // two boxes of 64 rows: MN-major tile
              tc::tma_load_3d(st, ma, &full[s], w.m0, kc, 0);
              tc::tma_load_3d(st + kGtMnAtom, ma, &full[s], w.m0 + kGtMnBox, kc, 0);
            } else {
              tc::tma_load_3d(st, ma, &full[s], kc, w.m0, 0);
            }
            if (w.mn & 2) {
              tc::tma_load_3d(st + P * Cfg::A_TILE, mb, &full[s], w.n0, kc, 0);
              tc::tma_load_3d(st + P * Cfg::A_TILE + kGtMnAtom, mb, &full[s], w.n0 + kGtMnBox, kc, 0);
            } else {
              tc::tma_load_3d(st + P * Cfg::A_TILE, mb, &full[s], kc, w.n0, 0);
            }
          }
        }
        if (!ok) break;
      }
      // drain: every copy this thread issued has landed before the CTA exits
      for (uint32_t j = it > uint32_t(S) ? it - S : 0u; j < it; ++j)
        if (!tc::mbar_wait(&full[j % S], (j / S) & 1)) {
          atomicExch(err, kErrGtDrain);
          break;
        }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer --
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(kGtBM, kGtBN);
      constexpr uint32_t idesc2 = tc::idesc_bf16_f32(kGtBM, 2 * kGtBN);
      uint32_t it = 0, g = 0;
      bool ok = true;
      for (uint32_t i = 0; ok; ++i) {
        const int r = i % kGtRing;
        if (!tc::mbar_wait(&wfull[r], (i / kGtRing) & 1)) {
          atomicExch(err, kErrGtMma);
          break;
        }
        const GtWork w = ring[r];
        tc::mbar_arrive(&wempty[r]);
        if (w.prob < 0) break;
        const int nch = (w.nk + CHUNK - 1) / CHUNK;
        for (int c = 0; c < nch && ok; ++c, ++g) {
          const int b = g % NACC;
          if (!tc::mbar_wait(&tempty[b], ((g / NACC) & 1) ^ 1)) {
            atomicExch(err, kErrGtMma);
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t acc = tmem + uint32_t(b * Cfg::ACC);
          const int kb1 = min(w.nk, (c + 1) * CHUNK);
          for (int kb = c * CHUNK; kb < kb1; ++kb, ++it) {
            const int s = it % S;
            if (!tc::mbar_wait(&full[s], (it / S) & 1)) {
              atomicExch(err, kErrGtMma);
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint8_t* st = smem + s * Cfg::STAGE;
            auto desc = [](uint32_t a) {
              return Cfg::BK == 64 ? tc::sdesc_kmajor_sw128(a) : tc::sdesc_kmajor_sw64(a);
            };
            if constexpr (P == 1) {
              // K = 16 per MMA: +32 bytes in a K-major swizzled row, +2 8-row
              // groups (2048 bytes) in an MN-major tile
              const uint32_t sa = tc::smem_u32(st), sb = tc::smem_u32(st + Cfg::A_TILE);
              const bool amn = w.mn & 1, bmn = w.mn & 2;
              const uint64_t ad = amn ? tc::sdesc_mn_sw128<kGtMnLbo, kGtMnSbo>(sa) : desc(sa);
              const uint64_t bd = bmn ? tc::sdesc_mn_sw128<kGtMnLbo, kGtMnSbo>(sb) : desc(sb);
              const uint64_t astep = amn ? (2048 >> 4) : 2, bstep = bmn ? (2048 >> 4) : 2;
              const uint32_t id = idesc | (amn ? 1u << 15 : 0u) | (bmn ? 1u << 16 : 0u);
#pragma unroll
              for (int j = 0; j < Cfg::BK / 16; ++j)
                tc::mma_bf16(acc, ad + astep * j, bd + bstep * j, id, kb != c * CHUNK || j != 0);
            } else if constexpr (P == 2) {
#pragma unroll
              for (int q = 0; q < Cfg::NPAIRS; ++q) {  // (0,0) (0,1) (1,0)
                const int pa = q == 2 ? 1 : 0, pb = q == 1 ? 1 : 0;
                const uint64_t ad = desc(tc::smem_u32(st + pa * Cfg::A_TILE));
                const uint64_t bd = desc(tc::smem_u32(st + P * Cfg::A_TILE + pb * Cfg::B_TILE));
#pragma unroll
                for (int j = 0; j < Cfg::BK / 16; ++j)  // K = 16 per MMA: +32 bytes in the swizzled row
                  tc::mma_bf16(acc, ad + 2 * j, bd + 2 * j, idesc, kb != c * CHUNK || q != 0 || j != 0);
              }
            } else {
              // P = 3: the B terms are adjacent 128-row tiles, so B terms
              // (0, 1) form one 256-row operand.  a(0) x [b0; b1] fills both
              // column halves (the first MMA of a chunk initialises both),
              // a(1) x [b0; b1] adds to both, a(0) b(2) and a(2) b(0) go to the
              // second half: the six products in four MMAs, the leading ones
              // kept apart from the small cross terms.
              const uint32_t sa = tc::smem_u32(st), sb = tc::smem_u32(st + P * Cfg::A_TILE);
              const uint64_t a0 = desc(sa), a1 = desc(sa + Cfg::A_TILE), a2 = desc(sa + 2 * Cfg::A_TILE);
              const uint64_t b01 = desc(sb), b2 = desc(sb + 2 * Cfg::B_TILE);
              const uint32_t acc2 = acc + uint32_t(kGtBN);
#pragma unroll
              for (int j = 0; j < Cfg::BK / 16; ++j) {  // K = 16 per MMA: +32 bytes in the swizzled row
                tc::mma_bf16(acc, a0 + 2 * j, b01 + 2 * j, idesc2, kb != c * CHUNK || j != 0);
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
    }
  } else {
    // ------------------------------------------------------------ epilogue --
    // warp w owns TMEM lanes [32*(w%4), +32) (one output row per thread) and
    // columns [64*h, +64), h = (w - 3) / 4
    const int q = warp & 3, h = (warp - 3) >> 2;
    uint32_t g = 0;
    for (uint32_t i = 0;; ++i) {
      const int r = i % kGtRing;
      if (!tc::mbar_wait(&wfull[r], (i / kGtRing) & 1)) {
        if (lane == 0) atomicExch(err, kErrGtEpilogue);
        break;
      }
      const GtWork w = ring[r];
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&wempty[r]);
      if (w.prob < 0) break;
      float sum[64];
#pragma unroll
      for (int j = 0; j < 64; ++j) sum[j] = 0.f;
      const int nch = (w.nk + CHUNK - 1) / CHUNK;
      bool ok = true;
      for (int c = 0; c < nch; ++c, ++g) {
        const int b = g % NACC;
        if (!tc::mbar_wait(&tfull[b], (g / NACC) & 1)) {
          if (lane == 0) atomicExch(err, kErrGtEpilogue);
          ok = false;
          break;
        }
        tc::tc_fence_after();
#pragma unroll
        for (int part = 0; part < Cfg::ACC / kGtBN; ++part)  // column halves fold onto the same sums
#pragma unroll
          for (int c0 = 0; c0 < 64; c0 += 32) {
            uint32_t v[32];
            tc::tmem_ld_32x32b_x32(
                tmem + (uint32_t(q * 32) << 16) + uint32_t(b * Cfg::ACC + part * kGtBN + h * 64 + c0), v);
            tc::tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 32; ++j) sum[c0 + j] += __uint_as_float(v[j]);
          }
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&tempty[b]);
      }
      if (!ok) break;
      if (w.splits > 1) {
        // the same sub-blocks are skipped in every slice of the tile
        if (w.m0 + q * 32 >= w.m || w.n0 + h * 64 >= w.n) continue;
        // whole 32 x 64 partials, columns and rows beyond the problem
        // included: unpredicated, the 64 loads of a slice are issued
        // together (the slots are allocated in full, the extra values unused)
        const int sub = h * 4 + q;
        constexpr int64_t kSlot = int64_t(kGtSubs) * kGtSubFloats;  // floats per slice
        float* const base = w.part + int64_t(sub) * kGtSubFloats + lane;
        {
          float* mine = base + int64_t(w.slice) * kSlot;
#pragma unroll
          for (int j = 0; j < 64; ++j) __stcg(mine + j * 32, sum[j]);
        }
        // climb the fold tree while this warp completes the node above it;
        // sum holds the value of node idx of the current level
        int idx = w.slice, nodes = w.splits, node_off = 0;
        int64_t span = 1;  // slices per node of the current level
        bool root = false;
        for (;;) {
          const int parent = idx / kGtFoldFan, first = parent * kGtFoldFan;
          const int nchild = min(kGtFoldFan, nodes - first);
          const int up = (nodes + kGtFoldFan - 1) / kGtFoldFan;
          unsigned int* t = w.tick + int64_t(node_off + parent) * kGtSubs + sub;
          __threadfence();
          __syncwarp();
          unsigned last = 0;
          if (lane == 0) last = atomicAdd(t, 1u) == unsigned(nchild - 1) ? 1u : 0u;
          if (__shfl_sync(0xffffffffu, last, 0) == 0u) break;
          __threadfence();
          if (lane == 0) *t = 0u;
          // a lone child already holds the node's value (and its slot holds it)
          if (nchild > 1) {
            const float* src = base + int64_t(first) * span * kSlot;
#pragma unroll
            for (int j = 0; j < 64; ++j) sum[j] = __ldcg(src + j * 32);
            for (int ch = 1; ch < nchild; ++ch) {
              src += span * kSlot;
#pragma unroll
              for (int j = 0; j < 64; ++j) sum[j] += __ldcg(src + j * 32);
            }
          }
          idx = parent;
          nodes = up;
          node_off += up;
          span *= kGtFoldFan;
          if (nodes == 1) {
            root = true;
            break;
          }
          if (nchild > 1) {
            float* dst = base + int64_t(idx) * span * kSlot;
#pragma unroll
            for (int j = 0; j < 64; ++j) __stcg(dst + j * 32, sum[j]);
          }
        }
        if (!root) continue;
      }
      const int64_t gm = int64_t(w.m0) + q * 32 + lane;
      if (gm < w.m) {
        float* const c = w.c;
        const int64_t ldc = w.ldc;
        const float alpha = w.alpha, beta = w.beta;
        const int nleft = w.n - w.n0 - h * 64;
        float* const cp = c + gm + (int64_t(w.n0) + h * 64) * ldc;
        // C is read 32 columns at a time, all loads before any store, so the
        // loads overlap (a store may alias a later load when ldc == 0)
#pragma unroll
        for (int j0 = 0; j0 < 64; j0 += 32) {
          float cv[32];
          if (beta != 0.f) {
#pragma unroll
            for (int j = 0; j < 32; ++j) cv[j] = (j0 + j < nleft) ? cp[int64_t(j0 + j) * ldc] : 0.f;
          }
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            if (j0 + j < nleft) {
              float v = alpha * sum[j0 + j];
              if (beta != 0.f) v = fmaf(beta, cv[j], v);
              cp[int64_t(j0 + j) * ldc] = v;
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
  if (threadIdx.x == 0) {
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

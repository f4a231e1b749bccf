// stream_sweep.cuh — TMA-fed versions of the two column-major matrix sweeps
// (see matvec.cuh for the math and the split / last-CTA combine).
//
// A dedicated producer warp streams 16 KB tiles of A into a ring of shared
// memory stages with 2-D tensor-map copies (cp.async.bulk.tensor, mbarrier
// completion); eight consumer warps fold them.  The bytes in flight per SM
// are then set by the ring (3 CTAs x 4 stages x 16 KB), not by registers,
// which is what keeps an HBM-bound sweep near the copy roofline.  Used when
// lda and the base pointer meet the tensor-map alignment rules (16-byte
// aligned base, lda * sizeof(T) a multiple of 16); the register-streaming
// kernels of matvec.cuh handle every other layout.
//
// Tiles that overhang the matrix are zero-filled by the copy engine; the
// consumers still mask rows >= M, columns outside their split and rows
// outside their chunk, so operators other than Add (Max, Min, Product) see
// only real elements.
#pragma once

#include "matvec.cuh"
#include "tc_ptx.cuh"

namespace gb {

constexpr int kStStages = 4;
constexpr int kStConsumers = 8;                       // consumer warps
constexpr int kStThreads = (kStConsumers + 1) * 32;   // + one producer warp
constexpr int kStTileBytes = 16384;

enum : int { kErrSweepFull = 201, kErrSweepEmpty = 202, kErrSweepDrain = 203, kErrSweepX = 204 };

// x elements staged in shared memory by the rows sweep (one column split)
constexpr int64_t kRowsXStage = 8192;
// bytes of x a cols-sweep CTA stages in shared memory (one row chunk's x)
constexpr int64_t kColsXBytes = 16384;

// barrier among the 8 consumer warps only (the producer keeps streaming)
__device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int32_t c0,
                                            int32_t c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(tc::smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(tc::smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

// Staging of x (n elements from src with stride inc) into shared memory xs,
// zero-filled up to `fill` elements.  With unit stride and a 16-byte-aligned
// src the 16-byte-aligned bulk of x is one cp.async.bulk copy issued by the
// producer warp at kernel start (so it travels with the first tiles of A);
// the consumers copy the rest with several loads in flight per thread.
template <typename T>
struct XStage {
  int64_t n, fill, inc;
  const T* src;
  uint32_t bulk;  // elements covered by the bulk copy (0: none)
  __device__ XStage(const T* src_, int64_t n_, int64_t fill_, int64_t inc_) : n(n_), fill(fill_), inc(inc_), src(src_) {
    constexpr int64_t V = 16 / int64_t(sizeof(T));
    const bool ok = inc == 1 && (reinterpret_cast<uintptr_t>(src) & 15) == 0;
    bulk = ok ? uint32_t(n / V * V) : 0u;
  }
  // producer lane: issue the bulk part
  __device__ void issue(T* xs, uint64_t* bar) const {
    if (bulk == 0) return;
    tc::mbar_arrive_expect_tx(bar, bulk * uint32_t(sizeof(T)));
    tc::bulk_load_1d(xs, src, bulk * uint32_t(sizeof(T)), bar);
  }
  // consumer threads (tid in [0, nthreads)): the rest, then wait for the bulk
  // part; false if that wait gave up
  template <int NTHREADS>
  __device__ bool finish(T* xs, uint64_t* bar, int tid) const {
    constexpr int U = 4;
    for (int64_t b = int64_t(bulk); b < fill; b += int64_t(U) * NTHREADS) {
      T v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = b + tid + int64_t(u) * NTHREADS;
        v[u] = i < n ? src[i * inc] : T(0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = b + tid + int64_t(u) * NTHREADS;
        if (i < fill) xs[i] = v[u];
      }
    }
    return bulk == 0 || tc::mbar_wait(bar, 0);
  }
};

// Producer loop shared by both sweeps: tile t of `ntiles` at coordinates
// (x0 + t*dx, y0 + t*dy).  Returns after every issued copy has landed.
template <int BOX_BYTES>
__device__ __forceinline__ void sweep_producer(const CUtensorMap* map, uint8_t* ring, uint64_t* full,
                                               uint64_t* empty, int ntiles, int32_t x0, int32_t dx, int32_t y0,
                                               int32_t dy, int* err) {
  tc::tma_prefetch_desc(map);
  int issued = 0;
  for (int t = 0; t < ntiles; ++t) {
    const int s = t % kStStages;
    const uint32_t ph = (t / kStStages) & 1;
    if (!tc::mbar_wait(&empty[s], ph ^ 1)) {
      atomicExch(err, kErrSweepEmpty);
      break;
    }
    tc::mbar_arrive_expect_tx(&full[s], BOX_BYTES);
    tma_load_2d(ring + s * kStTileBytes, map, &full[s], x0 + t * dx, y0 + t * dy);
    issued = t + 1;
  }
  for (int t = issued > kStStages ? issued - kStStages : 0; t < issued; ++t)
    if (!tc::mbar_wait(&full[t % kStStages], (t / kStStages) & 1)) {
      atomicExch(err, kErrSweepDrain);
      break;
    }
}

// ------------------------------------------------------------ rows sweep --
// CTA: BM rows (512 bytes) x one column split; tile = BM x 32 columns.
// Consumer warp w folds columns w, w+8, w+16, w+24 of each tile; lane l owns
// rows l*RPT .. l*RPT+RPT-1 (one 128-bit shared load per column).
template <class P, typename T, bool HAS_X>
__global__ void __launch_bounds__(kStThreads)
    rows_sweep_tma(const __grid_constant__ CUtensorMap tmA, P pol, int64_t M, int64_t N, const T* __restrict__ xb,
                   int64_t incx, int64_t cols_per_split, typename P::Acc* __restrict__ partials,
                   unsigned int* __restrict__ tickets, int* __restrict__ err) {
  pdl_trigger();
  using Acc = typename P::Acc;
  constexpr int RPT = Pack16<T>::n;
  constexpr int BM = 32 * RPT;
  constexpr int BC = kStTileBytes / (BM * int(sizeof(T)));  // 32
  extern __shared__ uint8_t smem_raw[];
  uint8_t* ring = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  uint64_t* full = reinterpret_cast<uint64_t*>(ring + kStStages * kStTileBytes);
  uint64_t* empty = full + kStStages;
  uint64_t* xbar = empty + kStStages;
  Acc* red = reinterpret_cast<Acc*>(xbar + 1);  // [kStConsumers][BM]
  T* xs = reinterpret_cast<T*>((reinterpret_cast<uintptr_t>(red + kStConsumers * BM) + 15) &
                               ~uintptr_t(15));  // [cols_per_split] when staged
  __shared__ bool is_last;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t rblock = blockIdx.x;
  const int64_t r0 = rblock * BM;
  const int64_t c0 = int64_t(blockIdx.y) * cols_per_split;
  const int64_t c1 = min(N, c0 + cols_per_split);
  const int ntiles = int(cdiv(c1 - c0, BC));
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStStages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], kStConsumers);
    }
    tc::mbar_init(xbar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  pdl_wait();  // A, x, the partials and the tickets belong to earlier kernels on the stream

  // x of this column split goes to shared memory while the first tiles land
  const bool xstaged = HAS_X && cols_per_split <= kRowsXStage;
  const XStage<T> xst(HAS_X ? xb + c0 * incx : xb, c1 - c0, c1 - c0, incx);
  if (warp == kStConsumers) {
    if (lane == 0) {
      if (xstaged) xst.issue(xs, xbar);
      sweep_producer<kStTileBytes>(&tmA, ring, full, empty, ntiles, int32_t(r0), 0, int32_t(c0), BC, err);
    }
  } else {
    bool ok = true;
    if (xstaged) {
      ok = xst.template finish<kStConsumers * 32>(xs, xbar, threadIdx.x);
      if (!ok && threadIdx.x == 0) atomicExch(err, kErrSweepX);
      consumers_sync();
    }
    Acc acc[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) acc[r] = pol.init();
    for (int t = 0; t < (ok ? ntiles : 0); ++t) {
      const int s = t % kStStages;
      if (!tc::mbar_wait(&full[s], (t / kStStages) & 1)) {
        if (lane == 0) atomicExch(err, kErrSweepFull);
        break;
      }
      const T* tile = reinterpret_cast<const T*>(ring + s * kStTileBytes);
      const int64_t cbase = c0 + int64_t(t) * BC;
#pragma unroll
      for (int u = 0; u < BC / kStConsumers; ++u) {
        const int jj = warp + u * kStConsumers;
        const int64_t gc = cbase + jj;
        if (gc < c1) {
          T v[RPT];
          Pack16<T>::get(*reinterpret_cast<const typename Pack16<T>::V*>(tile + jj * BM + lane * RPT), v);
          const T xv = HAS_X ? (xstaged ? xs[gc - c0] : xb[gc * incx]) : T(1);
#pragma unroll
          for (int r = 0; r < RPT; ++r) pol.add(acc[r], v[r], xv);
        }
      }
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&empty[s]);
    }
#pragma unroll
    for (int r = 0; r < RPT; ++r) red[warp * BM + lane * RPT + r] = acc[r];
  }
  __syncthreads();
  const int t = threadIdx.x;
  const int64_t row = r0 + t;
  Acc sacc;
  if (t < BM) {
    sacc = red[t];
#pragma unroll
    for (int w = 1; w < kStConsumers; ++w) pol.merge(sacc, red[w * BM + t]);
  }
  if (gridDim.y == 1) {
    if (t < BM && row < M) pol.finish(sacc, row);
    return;
  }
  if (t < BM && row < M) partials[int64_t(blockIdx.y) * M + row] = sacc;
  __threadfence();
  __syncthreads();
  if (t == 0) is_last = atomicAdd(tickets + rblock, 1u) == gridDim.y - 1;
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (t < BM && row < M) {
    Acc f = ldcg_any(partials + row);
    for (unsigned sp = 1; sp < gridDim.y; ++sp) pol.merge(f, ldcg_any(partials + int64_t(sp) * M + row));
    pol.finish(f, row);
  }
  if (t == 0) tickets[rblock] = 0u;
}

// ------------------------------------------------------------ cols sweep --
// CTA: a range of consecutive 16-column tiles x one chunk of rows; each tile
// is BR rows (1 KB) x 16 columns and the producer streams the chunk's row
// tiles of each column tile in turn.  The column tiles are dealt out in
// gridDim.x ranges that differ by at most one tile (range b starts at tile
// b * coltiles / gridDim.x), so a grid of exactly one wave is balanced.  Consumer warp w folds columns 2w and 2w+1 of
// a tile; lane l reads rows l*RPT + {0, 32*RPT} (two 128-bit shared loads
// per column) and the matching x from the chunk's copy of x in shared memory
// (staged once per CTA while the first tiles land).
template <class P, typename T, bool HAS_X>
__global__ void __launch_bounds__(kStThreads)
    cols_sweep_tma(const __grid_constant__ CUtensorMap tmA, P pol, int64_t M, int64_t N, const T* __restrict__ xb,
                   int64_t incx, int64_t rows_per_split, typename P::Acc* __restrict__ partials,
                   unsigned int* __restrict__ tickets, int* __restrict__ err) {
  pdl_trigger();
  using Acc = typename P::Acc;
  constexpr int RPT = Pack16<T>::n;
  constexpr int BR = 64 * RPT;                                  // 1 KB of rows
  constexpr int BC = kStTileBytes / (BR * int(sizeof(T)));      // 16 columns
  constexpr int CPW = BC / kStConsumers;                        // 2 columns per warp
  extern __shared__ uint8_t smem_raw[];
  uint8_t* ring = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  uint64_t* full = reinterpret_cast<uint64_t*>(ring + kStStages * kStTileBytes);
  uint64_t* empty = full + kStStages;
  uint64_t* xbar = empty + kStStages;
  T* xs = reinterpret_cast<T*>(xbar + 2);  // [rows_per_split] when HAS_X (16-byte aligned)
  __shared__ unsigned long long last_mask;  // bit c: this CTA folds column tile ct0 + c

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t coltiles = cdiv(N, BC);
  const int64_t ct0 = int64_t(blockIdx.x) * coltiles / gridDim.x;  // first column tile of this CTA
  const int nct = int((int64_t(blockIdx.x) + 1) * coltiles / gridDim.x - ct0);
  const int64_t r0 = int64_t(blockIdx.y) * rows_per_split;
  const int64_t rlen = min(M - r0, rows_per_split);
  const int nrt = int(cdiv(rlen, BR));  // row tiles per column tile
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStStages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], kStConsumers);
    }
    tc::mbar_init(xbar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  pdl_wait();  // A, x, the partials and the tickets belong to earlier kernels on the stream

  // the chunk's x (zero past the matrix) is staged while the first tiles land
  const XStage<T> xst(HAS_X ? xb + r0 * incx : xb, rlen, int64_t(nrt) * BR, incx);
  if (warp == kStConsumers) {
    if (lane == 0) {
      if (HAS_X) xst.issue(xs, xbar);
      // tile t: column tile t / nrt, row tile t % nrt
      tc::tma_prefetch_desc(&tmA);
      const int ntiles = nct * nrt;
      int issued = 0;
      for (int t = 0; t < ntiles; ++t) {
        const int s = t % kStStages;
        if (!tc::mbar_wait(&empty[s], ((t / kStStages) & 1) ^ 1)) {
          atomicExch(err, kErrSweepEmpty);
          break;
        }
        tc::mbar_arrive_expect_tx(&full[s], kStTileBytes);
        tma_load_2d(ring + s * kStTileBytes, &tmA, &full[s], int32_t(r0 + int64_t(t % nrt) * BR),
                    int32_t((ct0 + t / nrt) * BC));
        issued = t + 1;
      }
      for (int t = issued > kStStages ? issued - kStStages : 0; t < issued; ++t)
        if (!tc::mbar_wait(&full[t % kStStages], (t / kStStages) & 1)) {
          atomicExch(err, kErrSweepDrain);
          break;
        }
    }
  } else {
    bool ok = true;
    if (HAS_X) {
      ok = xst.template finish<kStConsumers * 32>(xs, xbar, threadIdx.x);
      if (!ok && threadIdx.x == 0) atomicExch(err, kErrSweepX);
      consumers_sync();
    }
    for (int c = 0; c < nct && ok; ++c) {
      Acc acc[CPW];
#pragma unroll
      for (int q = 0; q < CPW; ++q) acc[q] = pol.init();
      for (int rt = 0; rt < nrt; ++rt) {
        const int t = c * nrt + rt;
        const int s = t % kStStages;
        if (!tc::mbar_wait(&full[s], (t / kStStages) & 1)) {
          if (lane == 0) atomicExch(err, kErrSweepFull);
          ok = false;
          break;
        }
        const T* tile = reinterpret_cast<const T*>(ring + s * kStTileBytes);
        const int64_t roff = int64_t(rt) * BR;  // row offset within the chunk
        const bool full_tile = roff + BR <= rlen;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int rr = lane * RPT + h * 32 * RPT;
          T xv[RPT];
          if (HAS_X) Pack16<T>::get(*reinterpret_cast<const typename Pack16<T>::V*>(xs + roff + rr), xv);
#pragma unroll
          for (int q = 0; q < CPW; ++q) {
            const int jj = warp * CPW + q;
            T v[RPT];
            Pack16<T>::get(*reinterpret_cast<const typename Pack16<T>::V*>(tile + jj * BR + rr), v);
#pragma unroll
            for (int e = 0; e < RPT; ++e)
              if (full_tile || roff + rr + e < rlen) pol.add(acc[q], v[e], HAS_X ? xv[e] : T(1));
          }
        }
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&empty[s]);
      }
      if (!ok) break;
#pragma unroll
      for (int q = 0; q < CPW; ++q) {
        Acc a = acc[q];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) pol.merge(a, pol.shfl_down(a, off));
        const int64_t col = (ct0 + c) * BC + warp * CPW + q;
        if (lane == 0 && col < N) {
          if (gridDim.y == 1) pol.finish(a, col);
          else partials[int64_t(blockIdx.y) * N + col] = a;
        }
      }
    }
  }
  if (gridDim.y == 1) return;
  __threadfence();
  if (threadIdx.x == 0) last_mask = 0ull;
  __syncthreads();
  // the last CTA (over the row chunks) of each column tile folds its 16
  // columns; the tickets of all this CTA's tiles are taken at once (thread c
  // takes tile c), so the tail costs one round trip, not one per tile
  if (threadIdx.x < nct && atomicAdd(tickets + ct0 + threadIdx.x, 1u) == gridDim.y - 1)
    atomicOr(&last_mask, 1ull << threadIdx.x);
  __syncthreads();
  const unsigned long long mine = last_mask;
  if (mine == 0ull) return;
  __threadfence();
  for (int idx = threadIdx.x; idx < nct * BC; idx += blockDim.x) {
    const int c = idx / BC;
    const int64_t col = (ct0 + c) * BC + idx % BC;
    if (((mine >> c) & 1ull) && col < N) {
      Acc f = ldcg_any(partials + col);
      for (unsigned sp = 1; sp < gridDim.y; ++sp) pol.merge(f, ldcg_any(partials + int64_t(sp) * N + col));
      pol.finish(f, col);
    }
  }
  if (threadIdx.x < nct && ((mine >> threadIdx.x) & 1ull)) tickets[ct0 + threadIdx.x] = 0u;
}

// ------------------------------------------------------------------ host --
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn tensor_map_encoder();  // gemm_tc.cu

// Column-major M x N matrix, box = box_rows x box_cols, no swizzle.
template <typename T>
inline bool make_matrix_map(CUtensorMap* map, const T* base, int64_t M, int64_t N, int64_t lda, int box_rows,
                            int box_cols) {
  EncodeTiledFn fn = tensor_map_encoder();
  if (!fn) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) || ((lda * int64_t(sizeof(T))) & 15)) return false;
  if (M <= 0 || N <= 0 || M > (int64_t(1) << 31) || N > (int64_t(1) << 31)) return false;
  cuuint64_t dims[2] = {cuuint64_t(M), cuuint64_t(N)};
  cuuint64_t strides[1] = {cuuint64_t(lda * int64_t(sizeof(T)))};
  cuuint32_t box[2] = {cuuint32_t(box_rows), cuuint32_t(box_cols)};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2,
                  const_cast<T*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// Smem bytes of the two sweeps (ring + barriers + per-kernel extras + align slack).
template <typename Acc, typename T>
constexpr size_t rows_tma_smem(bool has_x) {
  return 128 + kStStages * kStTileBytes + (2 * kStStages + 1) * 8 +
         sizeof(Acc) * kStConsumers * 32 * (16 / sizeof(T)) + 16 + (has_x ? sizeof(T) * size_t(kRowsXStage) : 0);
}
template <typename T>
inline size_t cols_tma_smem(bool has_x, int64_t rows_per_split) {
  return 128 + kStStages * kStTileBytes + (2 * kStStages + 2) * 8 + (has_x ? sizeof(T) * size_t(rows_per_split) : 0);
}

struct TmaPlan {
  int64_t tiles, split, per_split;  // grid.x, grid.y, columns (rows sweep) or rows (cols sweep) per split
  bool full_wave;                   // the grid fills (nearly) every resident slot: launched early (PDL)
};

// rows sweep: first the split that fills one wave of 3 CTAs per SM; it is
// kept when its grid is resident at once with at least 2 CTAs on every SM
// (the resident CTAs per SM, at most 3, counted from the shared memory a CTA
// of that split takes, x staged or not).  Otherwise the split that
// minimises (waves of resident CTAs) x (tiles per CTA + 4): a last wave of
// few CTAs leaves HBM idle for the length of a whole CTA, and the 4 tiles
// stand for a CTA's start (ring fill, first-load latency).  GEMV 'n' GB/s,
// one-wave split -> this one (split in brackets): 16384^2 6139 (3: x staged,
// so 2 CTAs per SM and 1.26 waves) -> 6800 (14), 30000^2 3762 (1: 235 CTAs)
// -> 7140 (21), 40000 x 8192 5374 (1) -> 6876 (7); 8192^2 and the 16384^2
// outer reduction keep their one-wave splits (7 and 3; the cost rule's 7 for
// the reduction measured 1% slower).
constexpr int64_t kSmemPerSm = 233472;  // shared memory of one SM (sm_103a), bytes
constexpr int64_t kSmemPerCta = 1024;   // reserved by the system per resident CTA
constexpr int64_t kRowsMaxSplit = 64;

inline TmaPlan plan_rows_tma(int64_t M, int64_t N, int sm_count, int elem_bytes, int64_t smem_base, bool has_x) {
  const int64_t BM = 512 / elem_bytes, BC = kStTileBytes / 512;
  TmaPlan p;
  p.tiles = cdiv(M, BM);
  const int64_t ct = cdiv(N, BC);
  int64_t max_split = cdiv(N, 4 * BC);  // at least 4 tiles per CTA
  if (p.tiles > int64_t(kMaxTickets)) max_split = 1;
  if (max_split > kRowsMaxSplit) max_split = kRowsMaxSplit;
  // resident slots of a split of `per` tiles per CTA
  auto slots_of = [&](int64_t per) {
    const int64_t cols = per * BC;
    const int64_t smem = smem_base + ((has_x && cols <= kRowsXStage) ? elem_bytes * cols : 0);
    int64_t per_sm = kSmemPerSm / (smem + kSmemPerCta);
    if (per_sm > 3) per_sm = 3;
    if (per_sm < 1) per_sm = 1;
    return per_sm * sm_count;
  };
  int64_t s0 = 3 * int64_t(sm_count) / p.tiles;
  if (s0 > max_split) s0 = max_split;
  if (s0 < 1) s0 = 1;
  int64_t best_per = cdiv(ct, s0), best_slots = slots_of(best_per);
  const int64_t grid0 = p.tiles * cdiv(ct, best_per);
  if (!(grid0 <= best_slots && grid0 >= 2 * int64_t(sm_count))) {
    double best = -1.0;
    for (int64_t s = 1; s <= max_split; ++s) {
      const int64_t per = cdiv(ct, s), slots = slots_of(per);
      const double cost = double(cdiv(p.tiles * cdiv(ct, per), slots)) * double(per + 4);
      if (best < 0.0 || cost < best) {
        best = cost;
        best_per = per;
        best_slots = slots;
      }
    }
  }
  p.per_split = best_per * BC;
  p.split = cdiv(N, p.per_split);
  const int64_t grid = p.tiles * p.split;
  p.full_wave = grid <= best_slots && 32 * grid >= 31 * best_slots;
  return p;
}

// cols sweep: rows split into chunks (a multiple of the 1 KB tile; with x at
// most kColsXBytes of x per chunk so it fits in shared memory), then the
// column tiles are dealt out in `tiles` ranges per chunk, about `ctiles`
// each, so the grid is about one wave of resident CTAs (3 per SM with the
// 64 KB ring alone, 2 with x).  Finer row chunks (more CTAs, a full wave)
// were measured slower: their partial sums and the fold at the end cost
// more than the extra CTAs gain (GEMV 't' 8192^2 47.5 against 44.3 us).
inline TmaPlan plan_cols_tma(int64_t M, int64_t N, int sm_count, int elem_bytes, bool has_x) {
  const int64_t BR = 1024 / elem_bytes, BC = kStTileBytes / 1024;
  const int64_t slots = int64_t(sm_count) * (has_x ? 2 : 3);
  TmaPlan p;
  const int64_t coltiles = cdiv(N, BC);
  int64_t split = slots / coltiles;
  const int64_t min_split = has_x ? cdiv(M, kColsXBytes / elem_bytes) : 1;
  const int64_t max_split = cdiv(M, 4 * BR);
  if (split > max_split) split = max_split;
  if (split < min_split) split = min_split;
  if (split < 1) split = 1;
  p.per_split = cdiv(cdiv(M, split), BR) * BR;
  p.split = cdiv(M, p.per_split);
  // column tiles per CTA: enough CTAs for one wave, at least one tile each
  int64_t ctiles = cdiv(coltiles * p.split, slots);
  if (ctiles < 1) ctiles = 1;
  if (ctiles > 64) ctiles = 64;
  p.tiles = cdiv(coltiles, ctiles);
  p.full_wave = false;  // early launch (PDL) of a partial wave lands unevenly: measured slower
  return p;
}

// Launches the TMA rows sweep; returns false (nothing launched) when the
// layout does not qualify.
template <class P, typename T, bool HAS_X>
inline bool try_rows_sweep_tma(gbblas_handle_t h, const P& pol, int64_t M, int64_t N, const T* A, int64_t lda,
                               const T* xb, int64_t incx, gbblas_status_t* st) {
  using Acc = typename P::Acc;
  constexpr int BM = 512 / int(sizeof(T));
  constexpr int BC = kStTileBytes / 512;
  if (M < BM || N < 4 * BC) return false;
  TmaPlan p = plan_rows_tma(M, N, h->sm_count, int(sizeof(T)), int64_t(rows_tma_smem<Acc, T>(false)), HAS_X);
  if (p.split > 65535 || p.tiles > INT32_MAX) return false;
  CUtensorMap map;
  if (!make_matrix_map(&map, A, M, N, lda, BM, BC)) return false;
  Acc* partials = nullptr;
  if (p.split > 1) {
    void* tmp;
    *st = temp_acquire(h, sizeof(Acc) * p.split * M, &tmp);
    if (*st != GBBLAS_STATUS_SUCCESS) return true;
    partials = static_cast<Acc*>(tmp);
  }
  // x staged only when the split's columns fit the stage
  const size_t smem = rows_tma_smem<Acc, T>(false) +
                      ((HAS_X && p.per_split <= kRowsXStage) ? sizeof(T) * size_t(p.per_split) : 0);
  static std::atomic<uint64_t> attr{0};
  const cudaError_t ae = raise_smem_limit(attr, reinterpret_cast<const void*>(rows_sweep_tma<P, T, HAS_X>),
                                          int(rows_tma_smem<Acc, T>(HAS_X)), h->device);
  if (ae != cudaSuccess) {
    *st = cuda_fail(ae, "rows_sweep_tma: shared-memory limit");
    return true;
  }
  dim3 grid(unsigned(p.tiles), unsigned(p.split));
  const cudaError_t le = launch_pdl(p.full_wave, rows_sweep_tma<P, T, HAS_X>, grid, dim3(kStThreads), smem,
                                    h->stream, map, pol, M, N, xb, incx, p.per_split, partials, h->tickets,
                                    h->dev_error);
  *st = le != cudaSuccess ? cuda_fail(le, "rows_sweep_tma") : after_launch("rows_sweep_tma");
  return true;
}

template <class P, typename T, bool HAS_X>
inline bool try_cols_sweep_tma(gbblas_handle_t h, const P& pol, int64_t M, int64_t N, const T* A, int64_t lda,
                               const T* xb, int64_t incx, gbblas_status_t* st) {
  using Acc = typename P::Acc;
  constexpr int BR = 1024 / int(sizeof(T));
  constexpr int BC = kStTileBytes / 1024;
  if (M < 4 * BR || N < BC) return false;
  TmaPlan p = plan_cols_tma(M, N, h->sm_count, sizeof(T), HAS_X);
  if (p.tiles < 1 || p.split > 65535 || cdiv(N, BC) > int64_t(kMaxTickets) || p.tiles > INT32_MAX) return false;
  CUtensorMap map;
  if (!make_matrix_map(&map, A, M, N, lda, BR, BC)) return false;
  Acc* partials = nullptr;
  if (p.split > 1) {
    void* tmp;
    *st = temp_acquire(h, sizeof(Acc) * p.split * N, &tmp);
    if (*st != GBBLAS_STATUS_SUCCESS) return true;
    partials = static_cast<Acc*>(tmp);
  }
  const size_t smem = cols_tma_smem<T>(HAS_X, p.per_split);
  static std::atomic<uint64_t> attr{0};
  const cudaError_t ae = raise_smem_limit(attr, reinterpret_cast<const void*>(cols_sweep_tma<P, T, HAS_X>),
                                          int(cols_tma_smem<T>(HAS_X, kColsXBytes / int64_t(sizeof(T)))),
                                          h->device);
  if (ae != cudaSuccess) {
    *st = cuda_fail(ae, "cols_sweep_tma: shared-memory limit");
    return true;
  }
  dim3 grid(unsigned(p.tiles), unsigned(p.split));
  const cudaError_t le = launch_pdl(p.full_wave, cols_sweep_tma<P, T, HAS_X>, grid, dim3(kStThreads), smem,
                                    h->stream, map, pol, M, N, xb, incx, p.per_split, partials, h->tickets,
                                    h->dev_error);
  *st = le != cudaSuccess ? cuda_fail(le, "cols_sweep_tma") : after_launch("cols_sweep_tma");
  return true;
}

}  // namespace gb

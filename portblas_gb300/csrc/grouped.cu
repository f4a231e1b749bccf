// grouped.cu — grouped GEMM over uneven problems: a persistent launch with a
// device-side tile scheduler (preceded, on the tensor-core path, by one
// operand-conversion pass), captured once and replayed as a CUDA graph.
//
// portBLAS has only uniform batches (_gemm_batched / _gemm_strided_batched,
// src/interface/gemm_interface.hpp:200-240, with Gemm's batch loop in
// src/operations/blas3/gemm_local.hpp:438-516); each problem here keeps the
// blas::_gemm semantics (alpha/beta rules, any transposes, column-major).
//
// Scheduler: the problems are ordered by decreasing K per tile (longest tiles
// first, so the dynamic schedule ends balanced) and their tiles numbered in
// that order (prefix sums of per-problem tile counts in the device problem
// table; a tile -> problem table beside it).  Every CTA of a persistent grid
// (one per SM, at most one per tile) takes the next tile number from a global
// atomic counter, finds its problem, and computes the tile; no CTA ever waits
// on another.  The last CTA to finish resets the counters, so the same launch
// can be replayed from a CUDA graph with no host work.  On the tcgen05 path a
// problem whose tiles would outlast the mean work per SM gets split-K: its
// K is cut into slices, each slice a tile of its own (plan_splits).
//
// Two tile methods: the tcgen05 path of grouped_tc.cuh (default: 128 x 128
// tiles, BF16-term operands streamed by per-operand TMA maps), and a SIMT
// path (GBBLAS_GROUPED_METHOD=simt: 64 x 64 tiles; A and B slabs, BK = 16,
// converted to FP32 as they are staged in shared memory, any transpose; each
// of 256 threads accumulates a 4x4 FP32 register tile).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "gemm_internal.cuh"
#include "grouped_tc.cuh"

namespace gb {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn tensor_map_encoder();  // gemm_tc.cu

struct GroupedProblem {
  int m, n, k;
  int ta, tb;
  int tiles_n;       // tiles along N
  int64_t tile_start;  // first global tile number of this problem
  float alpha, beta;
  const void* a;
  const void* b;
  float* c;
  int64_t lda, ldb, ldc;
  // split-K (tcgen05 tiles): K slices per output tile, k-blocks per slice,
  // and the problem's first partial float / ticket in the launch's arrays
  int splits, kbs;
  int64_t part_off, tick_off;
  int64_t src;  // index of the problem in the caller's arrays
  // tcgen05 tiles, BF16 in: bit 0 / bit 1 set when A / B is read in place
  // with its rows contiguous (MN-major shared-memory tiles)
  int mn;
};

constexpr int kGT = 64, kGK = 16, kGThreads = 256;

template <typename T>
__device__ __forceinline__ float to_f32(T v);
template <>
__device__ __forceinline__ float to_f32<float>(float v) { return v; }
template <>
__device__ __forceinline__ float to_f32<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename T>
__device__ void grouped_tile(const GroupedProblem& p, int tm, int tn, float (&As)[kGK][kGT + 4],
                             float (&Bs)[kGK][kGT + 4]) {
  const T* A = static_cast<const T*>(p.a);
  const T* B = static_cast<const T*>(p.b);
  const int m0 = tm * kGT, n0 = tn * kGT;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < p.k; k0 += kGK) {
    // stage A(m, k) and B(k, n) slabs: 64 x 16 each, 4 elements per thread
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int e = threadIdx.x + i * kGThreads;  // 0..1023
      int r, kk;
      // A: contiguous along m when not transposed, along k when transposed
      if (!p.ta) { r = e % kGT; kk = e / kGT; } else { kk = e % kGK; r = e / kGK; }
      const int gm = m0 + r, gk = k0 + kk;
      float va = 0.f;
      if (gm < p.m && gk < p.k) va = to_f32<T>(p.ta ? A[gk + int64_t(gm) * p.lda] : A[gm + int64_t(gk) * p.lda]);
      As[kk][r] = va;
      // B: contiguous along k when not transposed, along n when transposed
      if (!p.tb) { kk = e % kGK; r = e / kGK; } else { r = e % kGT; kk = e / kGT; }
      const int gn = n0 + r, gk2 = k0 + kk;
      float vb = 0.f;
      if (gn < p.n && gk2 < p.k) vb = to_f32<T>(p.tb ? B[gn + int64_t(gk2) * p.ldb] : B[gk2 + int64_t(gn) * p.ldb]);
      Bs[kk][r] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        a[i] = As[kk][ty * 4 + i];
        b[i] = Bs[kk][tx * 4 + i];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  // each column's 4 C values are loaded before its stores so the loads overlap
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gn = n0 + tx * 4 + j;
    if (gn >= p.n) continue;
    float cv[4];
    if (p.beta != 0.f) {
#pragma unroll
      for (int i = 0; i < 4; ++i) cv[i] = (m0 + ty * 4 + i < p.m) ? p.c[m0 + ty * 4 + i + int64_t(gn) * p.ldc] : 0.f;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int gm = m0 + ty * 4 + i;
      if (gm >= p.m) continue;
      float v = p.alpha * acc[i][j];
      if (p.beta != 0.f) v = fmaf(p.beta, cv[i], v);
      p.c[gm + int64_t(gn) * p.ldc] = v;
    }
  }
}

// counters[0] = next tile, counters[1] = CTAs finished
template <typename T>
__global__ void __launch_bounds__(kGThreads) grouped_gemm_kernel(const GroupedProblem* __restrict__ probs,
                                                                 int count, int64_t total_tiles,
                                                                 unsigned long long* __restrict__ counters) {
  __shared__ float As[kGK][kGT + 4];
  __shared__ float Bs[kGK][kGT + 4];
  __shared__ long long tile;
  __shared__ GroupedProblem prob;
  for (;;) {
    if (threadIdx.x == 0) tile = (long long)atomicAdd(&counters[0], 1ull);
    __syncthreads();
    const long long t = tile;
    if (t >= total_tiles) break;
    if (threadIdx.x == 0) {
      int lo = 0, hi = count - 1;  // last problem with tile_start <= t
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (probs[mid].tile_start <= t) lo = mid; else hi = mid - 1;
      }
      prob = probs[lo];
    }
    __syncthreads();
    const int local = int(t - prob.tile_start);
    grouped_tile<T>(prob, local / prob.tiles_n, local % prob.tiles_n, As, Bs);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned long long done = atomicAdd(&counters[1], 1ull);
    if (done == gridDim.x - 1) {  // every CTA has stopped taking tiles
      counters[0] = 0ull;
      counters[1] = 0ull;
      __threadfence();
    }
  }
}

}  // namespace gb

// A grouped plan: one device block holding the problem table, the tile ->
// problem table, the scheduler counters and (tcgen05 path) the operand tensor
// maps, the operand conversion list and the BF16 terms; plus the instantiated
// CUDA graph of the launch.
struct gbblas_grouped_plan_s {
  int dtype = 0;
  int method = 1;  // 1: tcgen05 tiles (128 x 128), 0: SIMT tiles (64 x 64)
  int count = 0;
  int64_t total_tiles = 0;
  int grid = 0;
  void* block = nullptr;  // owned device block (plans only)
  gb::GroupedProblem* table = nullptr;
  int* tile_prob = nullptr;
  unsigned long long* counters = nullptr;
  CUtensorMap* maps = nullptr;
  gb::GtOperand* ops = nullptr;
  int n_ops = 0;
  int2* ctas = nullptr;  // (operand, part) of each split-pass CTA
  int n_ctas = 0;
  float* parts = nullptr;         // split-K partial blocks
  unsigned int* ticks = nullptr;  // split-K tickets (zero between launches)
  cudaGraphExec_t exec = nullptr;
  int max_splits = 1;
  int device = 0;
  int* err = nullptr;  // device error word of the creating handle
};

using namespace gb;

template <typename T, int P>
static gbblas_status_t launch_grouped_tc(cudaStream_t s, gbblas_grouped_plan_s* p, int* err) {
  constexpr int kChunk = kGtChunkK / GtCfg<P>::BK;  // k-blocks per TMEM chunk
  if (p->n_ops > 0) {
    grouped_split_kernel<T, P><<<unsigned(p->n_ctas), 256, 0, s>>>(p->ops, p->ctas);
    GB_TRY(after_launch("grouped_split"));
  }
  static std::atomic<uint64_t> attr{0};
  GB_CUDA_TRY(raise_smem_limit(attr, reinterpret_cast<const void*>(grouped_tc_kernel<P, kChunk, GroupedProblem>),
                               GtCfg<P>::SMEM, p->device));
  grouped_tc_kernel<P, kChunk, GroupedProblem><<<p->grid, kGtThreads, GtCfg<P>::SMEM, s>>>(
      p->table, p->tile_prob, p->maps, p->total_tiles, p->counters, p->parts, p->ticks, err);
  return after_launch("grouped_tc");
}

static gbblas_status_t launch_grouped(cudaStream_t s, gbblas_grouped_plan_s* p, int* err) {
  if (p->method == 1)
    return p->dtype == GBBLAS_DTYPE_BF16 ? launch_grouped_tc<__nv_bfloat16, 1>(s, p, err)
                                         : launch_grouped_tc<float, 3>(s, p, err);
  if (p->dtype == GBBLAS_DTYPE_BF16)
    grouped_gemm_kernel<__nv_bfloat16><<<p->grid, kGThreads, 0, s>>>(p->table, p->count, p->total_tiles, p->counters);
  else
    grouped_gemm_kernel<float><<<p->grid, kGThreads, 0, s>>>(p->table, p->count, p->total_tiles, p->counters);
  return after_launch("grouped_gemm");
}

// Tile kernel of a grouped launch: tcgen05 unless GBBLAS_GROUPED_METHOD=simt.
static int grouped_method() {
  const char* e = std::getenv("GBBLAS_GROUPED_METHOD");
  return (e && std::strcmp(e, "simt") == 0) ? 0 : 1;
}

extern "C" gbblas_status_t gbblas_grouped_plan_destroy(gbblas_grouped_plan_t plan) {
  if (!plan) return GBBLAS_STATUS_SUCCESS;
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  if (plan->block) cudaFree(plan->block);
  delete plan;
  return GBBLAS_STATUS_SUCCESS;
}

// ------------------------------------------------------------ split-K plan --
// The persistent kernel hands out tiles longest first (list scheduling), so
// its makespan is at least the longest tile.  When one problem's tiles are
// much longer (in K) than the mean work per SM (a few tall-skinny or long-K
// problems), their K is cut into slices.  A tile of nk k-blocks cut into S
// slices costs about nk/S k-blocks for the last slice to finish plus, per
// level of the fold tree it then climbs, its partial store and ticket (2 f)
// and the reads of the node's children (f each), f = 2 k-blocks for BF16
// inputs and 1.5 for FP32 inputs (whose k-blocks carry six term products);
// the S of least cost is each problem's upper bound.  Slices stay at least
// kGtMinSliceK deep and S <= kGtMaxSplits.  The launch is then kept within
// one wave of sm_count CTAs (more tiles than CTAs was measured slower: each
// extra round re-reads operand panels and the folds queue up) with slices of
// one common length L: S = ceil(nk / L) under that bound, L the shortest for
// which the tiles fit, an unsplit tile shorter than L counting as the
// fraction nk / L of a CTA (short tiles run on the CTAs the slices leave
// free, one after another).  Equal lengths rather than equal counts keep the
// longest problem from setting the makespan.
constexpr int kGtMaxSplits = 256;
constexpr int64_t kGtMinSliceK = 256;

// K slices of a tile of nk k-blocks under a cap of `cap` k-blocks per slice:
// splits >= 1 always (an empty K, alpha == 0, is one slice of nothing).
static void slice_shape(int64_t nk, int64_t cap, int& splits, int& kbs) {
  if (nk <= cap || nk <= 1 || cap < 1) {
    splits = 1;
    kbs = int(nk);
    return;
  }
  const int64_t sp = std::min<int64_t>(cdiv(nk, cap), kGtMaxSplits);
  const int64_t len = cdiv(nk, sp);
  splits = int(cdiv(nk, len));
  kbs = int(len);
}

// Cost in k-blocks of a tile of nk k-blocks in S slices (the rule above).
static double split_cost(int64_t nk, int64_t S, double f) {
  double t = double(cdiv(nk, S));
  for (int64_t n = S; n > 1; n = cdiv(n, kGtFoldFan)) t += f * double(std::min<int64_t>(n, kGtFoldFan) + 2);
  return t;
}

// Sets splits / kbs of every problem (k-blocks of `bk` elements; f as above).
static void plan_splits(std::vector<GroupedProblem>& tab, int bk, double fold_kb, int sm_count) {
  for (GroupedProblem& p : tab) {
    p.splits = 1;
    p.kbs = 0;
  }
  if (tab.empty() || sm_count <= 0) return;
  // GBBLAS_GROUPED_SPLITK: "0" never splits; N >= 2 cuts every problem of at
  // least N k-blocks into N slices (tuning); unset or "1": the rule above
  const char* env = std::getenv("GBBLAS_GROUPED_SPLITK");
  const long forced = env ? std::strtol(env, nullptr, 10) : 1;
  if (forced <= 0) return;
  if (forced >= 2) {
    for (GroupedProblem& p : tab) {
      const int64_t nkp = p.k > 0 ? cdiv(p.k, bk) : 0;
      if (nkp >= forced) slice_shape(nkp, cdiv(nkp, std::min<int64_t>(forced, kGtMaxSplits)), p.splits, p.kbs);
      if (p.splits == 1) p.kbs = 0;
    }
    return;
  }
  const size_t np = tab.size();
  std::vector<int64_t> out(np), nk(np), want(np, 1);
  int64_t work = 0, nk_max = 0;
  for (size_t i = 0; i < np; ++i) {
    out[i] = cdiv(tab[i].m, kGtBM) * tab[i].tiles_n;
    nk[i] = tab[i].k > 0 ? cdiv(tab[i].k, bk) : 0;
    work += out[i] * nk[i];
    nk_max = std::max(nk_max, nk[i]);
  }
  const int64_t min_kb = std::max<int64_t>(1, kGtMinSliceK / bk);
  // nothing to gain unless the longest tile is well above the mean load
  if (nk_max < 2 * min_kb || double(nk_max) <= 2.0 * double(work) / sm_count) return;
  std::vector<int64_t> best(np, 1);  // each problem's S of least cost
  for (size_t i = 0; i < np; ++i) {
    const int64_t smax = std::min<int64_t>({kGtMaxSplits, int64_t(sm_count), nk[i] / min_kb});
    double best_cost = split_cost(nk[i], 1, fold_kb);
    for (int64_t S = 2; S <= smax; ++S) {
      const double c = split_cost(nk[i], S, fold_kb);
      if (c < best_cost) {
        best_cost = c;
        best[i] = S;
      }
    }
  }
  // CTAs the launch occupies with slices of length L (k-blocks)
  auto slices_at = [&](int64_t L, size_t i) { return std::min<int64_t>(best[i], std::max<int64_t>(1, cdiv(nk[i], L))); };
  auto load_at = [&](int64_t L) {
    double t = 0.0;
    for (size_t i = 0; i < np; ++i) {
      const int64_t S = slices_at(L, i);
      t += double(out[i]) * (S > 1 ? double(S) : std::min(1.0, double(nk[i]) / double(L)));
    }
    return t;
  };
  // the shortest L that fits one wave (load_at does not grow with L)
  int64_t lo = 1, hi = std::max<int64_t>(1, nk_max);
  if (load_at(hi) > double(sm_count)) {
    lo = hi;  // even unsplit the tiles exceed one wave: no split
  } else {
    while (lo < hi) {
      const int64_t mid = lo + (hi - lo) / 2;
      if (load_at(mid) <= double(sm_count))
        hi = mid;
      else
        lo = mid + 1;
    }
  }
  for (size_t i = 0; i < np; ++i) want[i] = slices_at(lo, i);
  for (size_t i = 0; i < np; ++i) {
    if (want[i] > 1) slice_shape(nk[i], cdiv(nk[i], want[i]), tab[i].splits, tab[i].kbs);
    if (tab[i].splits == 1) tab[i].kbs = 0;
  }
}

// split_bk > 0: tcgen05 tiles with k-blocks of split_bk elements, split-K
// planned for sm_count SMs (split_p BF16 term products per element).
static gbblas_status_t build_table(int dtype, int64_t count, const char* transa, const char* transb,
                                   const int64_t* m, const int64_t* n, const int64_t* k, const float* alpha,
                                   const void* const* a, const int64_t* lda, const void* const* b,
                                   const int64_t* ldb, const float* beta, float* const* c, const int64_t* ldc,
                                   int tile_m, int tile_n, int split_bk, int split_p, int sm_count,
                                   std::vector<GroupedProblem>& tab, std::vector<int>& tile_prob, int64_t& tiles,
                                   int64_t& part_floats, int64_t& n_ticks) {
  if (dtype != GBBLAS_DTYPE_F32 && dtype != GBBLAS_DTYPE_BF16)
    return fail(GBBLAS_STATUS_UNSUPPORTED, "grouped: element type must be F32 or BF16");
  if (count < 0 || count > (1 << 24)) return fail(GBBLAS_STATUS_INVALID_ARG, "grouped: bad problem count");
  if (count > 0 && (!transa || !transb || !m || !n || !k || !alpha || !a || !lda || !b || !ldb || !beta || !c ||
                    !ldc))
    return fail(GBBLAS_STATUS_INVALID_ARG, "grouped: null host array");
  tab.clear();
  tab.reserve(size_t(count));
  tiles = 0;
  for (int64_t i = 0; i < count; ++i) {
    const char ca = char(transa[i] | 0x20), cb = char(transb[i] | 0x20);
    if (ca != 'n' && ca != 't' && ca != 'c') return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _TransA");
    if (cb != 'n' && cb != 't' && cb != 'c') return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _TransB");
    if (m[i] < 0 || n[i] < 0 || k[i] < 0 || m[i] > INT32_MAX || n[i] > INT32_MAX || k[i] > INT32_MAX)
      return fail(GBBLAS_STATUS_INVALID_ARG, "grouped: bad dimension");
    if (m[i] == 0 || n[i] == 0) continue;
    if (!c[i] || (k[i] > 0 && alpha[i] != 0.f && (!a[i] || !b[i])))
      return fail(GBBLAS_STATUS_INVALID_ARG, "grouped: null pointer");
    GroupedProblem p;
    p.m = int(m[i]);
    p.n = int(n[i]);
    // alpha == 0: C <- beta*C with A and B unread (gemm_interface.hpp:112-139)
    p.k = alpha[i] == 0.f ? 0 : int(k[i]);
    p.ta = ca != 'n';
    p.tb = cb != 'n';
    p.tiles_n = int(cdiv(n[i], tile_n));
    p.tile_start = 0;
    p.alpha = alpha[i];
    p.beta = beta[i];
    p.a = a[i];
    p.b = b[i];
    p.c = c[i];
    p.lda = lda[i];
    p.ldb = ldb[i];
    p.ldc = ldc[i];
    p.splits = 1;
    p.kbs = 0;
    p.part_off = 0;
    p.tick_off = 0;
    p.src = i;
    p.mn = 0;
    tab.push_back(p);
  }
  if (split_bk > 0) {
    // cost model per k-block: a BF16 k-block (one product) is ~3x shorter
    // than an FP32 one (six products), so the fixed costs weigh more
    plan_splits(tab, split_bk, split_p == 1 ? 2.0 : 1.5, sm_count);
  }
  // longest tiles (slices) first; tiles numbered in that order
  auto tile_k = [](const GroupedProblem& p, int bk) { return p.splits > 1 ? int64_t(p.kbs) * bk : int64_t(p.k); };
  std::stable_sort(tab.begin(), tab.end(), [&](const GroupedProblem& x, const GroupedProblem& y) {
    return tile_k(x, split_bk) > tile_k(y, split_bk);
  });
  tile_prob.clear();
  part_floats = 0;
  n_ticks = 0;
  for (size_t i = 0; i < tab.size(); ++i) {
    GroupedProblem& p = tab[i];
    p.tile_start = tiles;
    const int64_t out = cdiv(int64_t(p.m), tile_m) * p.tiles_n;
    const int64_t nt = out * p.splits;
    if (p.splits > 1) {
      p.part_off = part_floats;
      p.tick_off = n_ticks;
      part_floats += out * p.splits * kGtTileFloats;
      n_ticks += out * gt_fold_nodes(p.splits) * kGtSubs;
    }
    tiles += nt;
    tile_prob.insert(tile_prob.end(), size_t(nt), int(i));
  }
  return GBBLAS_STATUS_SUCCESS;
}

// MN-major in-place tiles for BF16 operands whose rows are contiguous
// (GBBLAS_GROUPED_MN=0 turns them off: such operands are then transposed by
// the conversion pass).
static bool mn_tiles_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("GBBLAS_GROUPED_MN");
    return !(v && v[0] == '0');
  }();
  return on;
}

// One operand of the tcgen05 path: converted into BF16 terms (offset into
// the term area) or, for a BF16 operand with a 16-byte-aligned base and
// leading dimension, mapped in place: K-contiguous (direct) or with its rows
// contiguous (mn: the tile kernel loads 64-row boxes into MN-major tiles).
// A BF16 operand with contiguous rows that TMA cannot address in place is
// copied (not transposed) by the pass into a 16-byte pitch and read as
// MN-major tiles from there (mn and !direct, Kp: the row pitch).
struct TcOperandPlan {
  int prob, which;  // which: 0 = A (rows m), 1 = B (rows n)
  bool direct, mn, copy;
  int64_t rows, k, sr, Kp;
  const void* src;
  size_t off;
  int64_t sk;
};

static void plan_tc_operands(int dtype, std::vector<GroupedProblem>& tab, std::vector<TcOperandPlan>& pl,
                             size_t& term_bytes) {
  const int P = dtype == GBBLAS_DTYPE_BF16 ? 1 : 3;
  pl.clear();
  term_bytes = 0;
  for (size_t i = 0; i < tab.size(); ++i) {
    GroupedProblem& p = tab[i];
    p.mn = 0;
    if (p.k == 0) continue;
    for (int which = 0; which < 2; ++which) {
      TcOperandPlan o{};
      o.prob = int(i);
      o.which = which;
      o.k = p.k;
      // A(m, k) = ta ? A[k + m*lda] : A[m + k*lda];  B as rows n: tb ? B[n + k*ldb] : B[k + n*ldb]
      int64_t sk;
      if (which == 0) {
        o.rows = p.m;
        o.sr = p.ta ? p.lda : 1;
        sk = p.ta ? 1 : p.lda;
        o.src = p.a;
      } else {
        o.rows = p.n;
        o.sr = p.tb ? 1 : p.ldb;
        sk = p.tb ? p.ldb : 1;
        o.src = p.b;
      }
      o.sk = sk;
      const bool al16 = (reinterpret_cast<uintptr_t>(o.src) & 15) == 0;
      o.direct = dtype == GBBLAS_DTYPE_BF16 && sk == 1 && o.sr % 8 == 0 && o.sr >= o.k && al16;
      const bool rows_contig = dtype == GBBLAS_DTYPE_BF16 && o.sr == 1 && sk != 1 && mn_tiles_enabled();
      o.mn = rows_contig && sk % 8 == 0 && sk >= o.rows && al16;
      o.copy = rows_contig && !o.mn;
      if (o.mn || o.copy) p.mn |= 1 << which;
      if (o.copy) {
        o.Kp = cdiv(o.rows, int64_t(16)) * 16;  // row pitch of the copy
        o.off = term_bytes;
        term_bytes += (size_t(o.Kp) * size_t(o.k) * 2 + 255) & ~size_t(255);
      } else if (!o.direct && !o.mn) {
        // FP32: k-block-major terms in 32-deep blocks (gt_term3_ptr)
        o.Kp = cdiv(o.k, int64_t(P == 3 ? 32 : 16)) * (P == 3 ? 32 : 16);
        o.off = term_bytes;
        term_bytes += (size_t(P) * size_t(o.rows) * size_t(o.Kp) * 2 + 255) & ~size_t(255);
        o.sr = which == 0 ? (p.ta ? p.lda : 1) : (p.tb ? 1 : p.ldb);
      }
      pl.push_back(o);
    }
  }
}

// Tensor maps (two per problem) and the conversion list, once the term area
// has its address.
static gbblas_status_t encode_tc_operands(int dtype, const std::vector<GroupedProblem>& tab,
                                          const std::vector<TcOperandPlan>& pl, uint8_t* terms,
                                          std::vector<CUtensorMap>& maps, std::vector<GtOperand>& ops,
                                          std::vector<int2>& ctas) {
  EncodeTiledFn fn = tensor_map_encoder();
  if (!fn) return fail(GBBLAS_STATUS_UNSUPPORTED, "grouped: cuTensorMapEncodeTiled unavailable");
  const int P = dtype == GBBLAS_DTYPE_BF16 ? 1 : 3;
  maps.assign(2 * std::max<size_t>(1, tab.size()), CUtensorMap{});
  ops.clear();
  for (const TcOperandPlan& o : pl) {
    const GroupedProblem& p = tab[size_t(o.prob)];
    void* base;
    cuuint64_t dims[3], strides[2];
    const int bk = dtype == GBBLAS_DTYPE_BF16 ? GtCfg<1>::BK : GtCfg<3>::BK;
    cuuint32_t box[3] = {cuuint32_t(bk), cuuint32_t(o.which == 0 ? kGtBM : kGtBN), 1};
    if (o.mn || o.copy) {
      // rows contiguous: boxes of 64 rows (128 bytes) x 64 k, two per tile,
      // in place or from the pass's copy
      const int64_t pitch = o.copy ? o.Kp : o.sk;
      base = o.copy ? static_cast<void*>(terms + o.off) : const_cast<void*>(o.src);
      dims[0] = cuuint64_t(o.rows);
      dims[1] = cuuint64_t(o.k);
      dims[2] = 1;
      strides[0] = cuuint64_t(pitch) * 2;
      strides[1] = cuuint64_t(pitch) * 2 * cuuint64_t(o.k);
      box[0] = cuuint32_t(kGtMnBox);
      box[1] = cuuint32_t(bk);
      if (o.copy) {
        // the copy is the pass's K-contiguous case with rows and K swapped:
        // line k (stride sk in the source) of `rows` contiguous elements
        GtOperand g;
        g.src = o.src;
        g.sr = o.sk;
        g.sk = 1;
        g.rows = int(o.k);
        g.K = int(o.rows);
        g.Kp = int(o.Kp);
        g.blocks = int(gt_split_blocks(o.k, o.Kp, true, true));
        g.parts = int(cdiv(int64_t(g.blocks), int64_t(kGtSplitTiles)));
        g.out = reinterpret_cast<__nv_bfloat16*>(terms + o.off);
        ops.push_back(g);
      }
    } else if (o.direct) {
      base = const_cast<void*>(o.src);
      dims[0] = cuuint64_t(o.k);
      dims[1] = cuuint64_t(o.rows);
      dims[2] = 1;
      strides[0] = cuuint64_t(o.sr) * 2;
      strides[1] = cuuint64_t(o.sr) * 2 * cuuint64_t(o.rows);
    } else {
      base = terms + o.off;
      if (P == 3) {
        // [Kp / 32][3][rows][32]: planes (k-block, term) of rows x 64 bytes
        dims[0] = cuuint64_t(bk);
        dims[1] = cuuint64_t(o.rows);
        dims[2] = cuuint64_t(P) * cuuint64_t(o.Kp / bk);
        strides[0] = cuuint64_t(bk) * 2;
        strides[1] = cuuint64_t(bk) * 2 * cuuint64_t(o.rows);
      } else {
        dims[0] = cuuint64_t(o.Kp);
        dims[1] = cuuint64_t(o.rows);
        dims[2] = cuuint64_t(P);
        strides[0] = cuuint64_t(o.Kp) * 2;
        strides[1] = cuuint64_t(o.Kp) * 2 * cuuint64_t(o.rows);
      }
      box[2] = cuuint32_t(P);
      GtOperand g;
      g.src = o.src;
      g.sr = o.sr;
      g.sk = o.which == 0 ? (p.ta ? 1 : p.lda) : (p.tb ? p.ldb : 1);
      g.rows = int(o.rows);
      g.K = int(o.k);
      g.Kp = int(o.Kp);
      g.blocks = int(gt_split_blocks(o.rows, o.Kp, g.sk == 1, P == 1));
      g.parts = int(cdiv(int64_t(g.blocks), int64_t(kGtSplitTiles)));
      g.out = reinterpret_cast<__nv_bfloat16*>(terms + o.off);
      ops.push_back(g);
    }
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(&maps[size_t(2 * o.prob + o.which)], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides,
                    box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
      return fail(GBBLAS_STATUS_UNSUPPORTED, "grouped: tensor map encode failed (" + std::to_string(int(r)) + ")");
  }
  // largest conversions first
  std::stable_sort(ops.begin(), ops.end(), [](const GtOperand& x, const GtOperand& y) { return x.blocks > y.blocks; });
  ctas.clear();
  for (size_t i = 0; i < ops.size(); ++i)
    for (int part = 0; part < ops[i].parts; ++part) ctas.push_back(make_int2(int(i), part));
  return GBBLAS_STATUS_SUCCESS;
}

static size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte layout of a launch's device block.
struct GroupedLayout {
  size_t table, tile_prob, counters, maps, ops, ctas, ticks, parts, terms, total;
};

static GroupedLayout grouped_layout(size_t count, size_t tiles, size_t n_maps, size_t n_ops, size_t n_ctas,
                                    size_t n_ticks, size_t part_floats, size_t term_bytes) {
  GroupedLayout L;
  L.table = 0;
  L.tile_prob = round256(sizeof(GroupedProblem) * std::max<size_t>(1, count));
  L.counters = L.tile_prob + round256(sizeof(int) * std::max<size_t>(1, tiles));
  L.maps = L.counters + 256;
  L.ops = L.maps + round256(sizeof(CUtensorMap) * n_maps);
  L.ctas = L.ops + round256(sizeof(GtOperand) * n_ops);
  L.ticks = L.ctas + round256(sizeof(int2) * n_ctas);
  L.parts = L.ticks + round256(sizeof(unsigned int) * n_ticks);
  L.terms = L.parts + round256(sizeof(float) * part_floats);
  L.total = L.terms + term_bytes;
  return L;
}

static int grouped_grid(gbblas_handle_t h, int64_t tiles, int method) {
  // resident CTAs per SM: SIMT 8 x 256 threads; tcgen05 one (shared memory)
  const int per_sm = method == 0 ? 8 : 1;
  const int64_t cap = int64_t(h->sm_count) * per_sm;
  return int(std::max<int64_t>(1, std::min<int64_t>(tiles, cap)));
}

// Builds everything a launch needs on the host, points `pl` into `block`
// (which must hold layout.total bytes) and returns the host images to upload.
struct GroupedHost {
  std::vector<GroupedProblem> tab;
  std::vector<int> tile_prob;
  std::vector<TcOperandPlan> operands;
  std::vector<CUtensorMap> maps;
  std::vector<GtOperand> ops;
  std::vector<int2> ctas;
  size_t term_bytes = 0;
  int64_t tiles = 0;
  int64_t part_floats = 0, n_ticks = 0;  // split-K
};

static GroupedLayout host_layout(const GroupedHost& H) {
  return grouped_layout(H.tab.size(), size_t(H.tiles), H.maps.size(), H.ops.size(), H.ctas.size(),
                        size_t(H.n_ticks), size_t(H.part_floats), H.term_bytes);
}

static GroupedLayout bind_plan(gbblas_handle_t h, int dtype, int method, GroupedHost& H, void* block,
                               gbblas_grouped_plan_s* pl) {
  GroupedLayout L = host_layout(H);
  uint8_t* b = static_cast<uint8_t*>(block);
  pl->dtype = dtype;
  pl->method = method;
  pl->count = int(H.tab.size());
  pl->total_tiles = H.tiles;
  pl->grid = grouped_grid(h, H.tiles, method);
  pl->table = reinterpret_cast<GroupedProblem*>(b + L.table);
  pl->tile_prob = reinterpret_cast<int*>(b + L.tile_prob);
  pl->counters = reinterpret_cast<unsigned long long*>(b + L.counters);
  pl->maps = method == 1 ? reinterpret_cast<CUtensorMap*>(b + L.maps) : nullptr;
  pl->ops = method == 1 ? reinterpret_cast<GtOperand*>(b + L.ops) : nullptr;
  pl->n_ops = method == 1 ? int(H.ops.size()) : 0;
  pl->ctas = method == 1 ? reinterpret_cast<int2*>(b + L.ctas) : nullptr;
  pl->n_ctas = method == 1 ? int(H.ctas.size()) : 0;
  pl->ticks = H.n_ticks > 0 ? reinterpret_cast<unsigned int*>(b + L.ticks) : nullptr;
  pl->parts = H.part_floats > 0 ? reinterpret_cast<float*>(b + L.parts) : nullptr;
  return L;
}

// Host-side preparation shared by plans and one-shot calls.  The term area's
// address is only known once the block exists, so the maps are encoded
// against `block` (may be null while sizing).
static gbblas_status_t prepare_host(gbblas_handle_t h, int dtype, int method, int64_t count, const char* transa,
                                    const char* transb, const int64_t* m, const int64_t* n, const int64_t* k,
                                    const float* alpha, const void* const* a, const int64_t* lda,
                                    const void* const* b, const int64_t* ldb, const float* beta, float* const* c,
                                    const int64_t* ldc, GroupedHost& H) {
  const bool bf16 = dtype == GBBLAS_DTYPE_BF16;
  const int split_bk = method == 1 ? (bf16 ? GtCfg<1>::BK : GtCfg<3>::BK) : 0;
  GB_TRY(build_table(dtype, count, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc,
                     method ? kGtBM : kGT, method ? kGtBN : kGT, split_bk, bf16 ? 1 : 3, h->sm_count, H.tab,
                     H.tile_prob, H.tiles, H.part_floats, H.n_ticks));
  if (method == 1) {
    plan_tc_operands(dtype, H.tab, H.operands, H.term_bytes);
    // sizes only: maps two per problem, one conversion per non-direct operand
    H.maps.assign(2 * std::max<size_t>(1, H.tab.size()), CUtensorMap{});
    size_t n_conv = 0, n_ctas = 0;
    for (const TcOperandPlan& o : H.operands)
      if (o.copy) {
        ++n_conv;
        n_ctas += size_t(cdiv(gt_split_blocks(o.k, o.Kp, true, true), int64_t(kGtSplitTiles)));
      } else if (!o.direct && !o.mn) {
        ++n_conv;
        n_ctas += size_t(cdiv(gt_split_blocks(o.rows, o.Kp, o.sk == 1, bf16), int64_t(kGtSplitTiles)));
      }
    H.ops.resize(n_conv);
    H.ctas.resize(n_ctas);
  }
  return GBBLAS_STATUS_SUCCESS;
}

static gbblas_status_t upload(const GroupedHost& H, const GroupedLayout& L, uint8_t* block, cudaStream_t s) {
  if (!H.tab.empty())
    GB_CUDA_TRY(cudaMemcpyAsync(block + L.table, H.tab.data(), sizeof(GroupedProblem) * H.tab.size(),
                                cudaMemcpyHostToDevice, s));
  if (!H.tile_prob.empty())
    GB_CUDA_TRY(cudaMemcpyAsync(block + L.tile_prob, H.tile_prob.data(), sizeof(int) * H.tile_prob.size(),
                                cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemsetAsync(block + L.counters, 0, 2 * sizeof(unsigned long long), s));
  if (H.n_ticks > 0) GB_CUDA_TRY(cudaMemsetAsync(block + L.ticks, 0, sizeof(unsigned int) * size_t(H.n_ticks), s));
  if (!H.maps.empty() && L.ops > L.maps)
    GB_CUDA_TRY(cudaMemcpyAsync(block + L.maps, H.maps.data(), sizeof(CUtensorMap) * H.maps.size(),
                                cudaMemcpyHostToDevice, s));
  if (!H.ops.empty())
    GB_CUDA_TRY(cudaMemcpyAsync(block + L.ops, H.ops.data(), sizeof(GtOperand) * H.ops.size(),
                                cudaMemcpyHostToDevice, s));
  if (!H.ctas.empty())
    GB_CUDA_TRY(cudaMemcpyAsync(block + L.ctas, H.ctas.data(), sizeof(int2) * H.ctas.size(),
                                cudaMemcpyHostToDevice, s));
  return GBBLAS_STATUS_SUCCESS;
}

extern "C" {

gbblas_status_t gbblas_grouped_plan_create(gbblas_handle_t h, int dtype, int64_t count, const char* transa,
                                           const char* transb, const int64_t* m, const int64_t* n,
                                           const int64_t* k, const float* alpha, const void* const* a,
                                           const int64_t* lda, const void* const* b, const int64_t* ldb,
                                           const float* beta, float* const* c, const int64_t* ldc,
                                           gbblas_grouped_plan_t* out) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "grouped: null handle");
  if (!out) return fail(GBBLAS_STATUS_INVALID_ARG, "grouped: null plan pointer");
  *out = nullptr;
  const int method = grouped_method();
  GroupedHost H;
  GB_TRY(prepare_host(h, dtype, method, count, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, H));
  auto* plan = new (std::nothrow) gbblas_grouped_plan_s();
  if (!plan) return fail(GBBLAS_STATUS_ALLOC_FAILED, "grouped: out of host memory");
  plan->err = h->dev_error;
  plan->device = h->device;
  const GroupedLayout L0 = host_layout(H);
  cudaError_t e = cudaMalloc(&plan->block, L0.total);
  if (e != cudaSuccess) {
    delete plan;
    return cuda_fail(e, "grouped: plan allocation");
  }
  const GroupedLayout L = bind_plan(h, dtype, method, H, plan->block, plan);
  gbblas_status_t st = GBBLAS_STATUS_SUCCESS;
  if (method == 1)
    st = encode_tc_operands(dtype, H.tab, H.operands, static_cast<uint8_t*>(plan->block) + L.terms, H.maps, H.ops,
                            H.ctas);
  if (st == GBBLAS_STATUS_SUCCESS) st = upload(H, L, static_cast<uint8_t*>(plan->block), h->stream);
  if (st == GBBLAS_STATUS_SUCCESS) {
    e = cudaStreamSynchronize(h->stream);  // the host images go out of scope
    if (e != cudaSuccess) st = cuda_fail(e, "grouped: plan upload");
  }
  if (st != GBBLAS_STATUS_SUCCESS) {
    gbblas_grouped_plan_destroy(plan);
    return st;
  }
  for (const GroupedProblem& p : H.tab) plan->max_splits = std::max(plan->max_splits, p.splits);
  *out = plan;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_grouped_schedule(int dtype, int64_t count, const char* transa, const char* transb,
                                        const int64_t* m, const int64_t* n, const int64_t* k, const float* alpha,
                                        int sm_count, int64_t* tiles, int* splits) {
  clear_error();
  if (sm_count < 1) return fail(GBBLAS_STATUS_INVALID_ARG, "grouped schedule: sm_count < 1");
  if (count < 0 || count > (1 << 24)) return fail(GBBLAS_STATUS_INVALID_ARG, "grouped: bad problem count");
  // the planner only looks at sizes: stand-in operands and scalars
  std::vector<const void*> ptr(size_t(count), reinterpret_cast<const void*>(uintptr_t(256)));
  std::vector<float*> cptr(size_t(count), reinterpret_cast<float*>(uintptr_t(256)));
  std::vector<float> zero(size_t(count), 0.f);
  std::vector<int64_t> ld(size_t(count), 1);
  for (int64_t i = 0; i < count && m && n && k; ++i) ld[size_t(i)] = std::max<int64_t>({1, m[i], n[i], k[i]});
  const bool bf16 = dtype == GBBLAS_DTYPE_BF16;
  std::vector<GroupedProblem> tab;
  std::vector<int> tile_prob;
  int64_t n_tiles = 0, part_floats = 0, n_ticks = 0;
  GB_TRY(build_table(dtype, count, transa, transb, m, n, k, alpha, ptr.data(), ld.data(), ptr.data(), ld.data(),
                     zero.data(), cptr.data(), ld.data(), kGtBM, kGtBN, bf16 ? GtCfg<1>::BK : GtCfg<3>::BK,
                     bf16 ? 1 : 3, sm_count, tab, tile_prob, n_tiles, part_floats, n_ticks));
  if (tiles) *tiles = n_tiles;
  if (splits) {
    for (int64_t i = 0; i < count; ++i) splits[i] = 0;  // empty problems (m or n == 0) have no tiles
    for (const GroupedProblem& p : tab) splits[p.src] = p.splits;
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_grouped_plan_info(gbblas_grouped_plan_t plan, int64_t* tiles, int* max_splits) {
  clear_error();
  if (!plan) return fail(GBBLAS_STATUS_INVALID_ARG, "grouped: null plan");
  if (tiles) *tiles = plan->total_tiles;
  if (max_splits) *max_splits = plan->max_splits;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_grouped_plan_run(gbblas_handle_t h, gbblas_grouped_plan_t plan) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "grouped: null handle");
  if (!plan) return fail(GBBLAS_STATUS_INVALID_ARG, "grouped: null plan");
  if (plan->device != h->device)
    return fail(GBBLAS_STATUS_INVALID_ARG, "grouped: the plan belongs to another device than the handle");
  if (plan->total_tiles == 0) return GBBLAS_STATUS_SUCCESS;
  if (!plan->exec) {
    // capture the launch once on a private stream (the handle's stream may be
    // the legacy default stream, which cannot be captured)
    cudaStream_t cs;
    GB_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      gbblas_status_t s = launch_grouped(cs, plan, plan->err);
      e = cudaStreamEndCapture(cs, &graph);
      if (s != GBBLAS_STATUS_SUCCESS && e == cudaSuccess) e = cudaErrorLaunchFailure;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&plan->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) {
      plan->exec = nullptr;
      return cuda_fail(e, "grouped: graph capture");
    }
  }
  GB_CUDA_TRY(cudaGraphLaunch(plan->exec, h->stream));
  return after_launch("grouped_gemm(graph)");
}

gbblas_status_t gbblas_gemm_grouped(gbblas_handle_t h, int dtype, int64_t count, const char* transa,
                                    const char* transb, const int64_t* m, const int64_t* n, const int64_t* k,
                                    const float* alpha, const void* const* a, const int64_t* lda,
                                    const void* const* b, const int64_t* ldb, const float* beta, float* const* c,
                                    const int64_t* ldc) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "grouped: null handle");
  const int method = grouped_method();
  GroupedHost H;
  GB_TRY(prepare_host(h, dtype, method, count, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, H));
  if (H.tiles == 0) return GBBLAS_STATUS_SUCCESS;
  // one-shot: the whole block lives in the handle's stream-ordered temp memory
  const GroupedLayout L0 = host_layout(H);
  void* ws = nullptr;
  GB_TRY(temp_acquire(h, L0.total, &ws));
  gbblas_grouped_plan_s tmp;
  tmp.device = h->device;
  const GroupedLayout L = bind_plan(h, dtype, method, H, ws, &tmp);
  if (method == 1)
    GB_TRY(encode_tc_operands(dtype, H.tab, H.operands, static_cast<uint8_t*>(ws) + L.terms, H.maps, H.ops, H.ctas));
  GB_TRY(upload(H, L, static_cast<uint8_t*>(ws), h->stream));
  gbblas_status_t s = launch_grouped(h->stream, &tmp, h->dev_error);
  // the host images (pageable) were staged by the copies before they returned
  return s;
}

}  // extern "C"

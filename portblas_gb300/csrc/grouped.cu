// grouped.cu — grouped GEMM over uneven problems: one persistent launch with
// a device-side tile scheduler, replayed through a CUDA graph.
//
// portBLAS has only uniform batches (_gemm_batched / _gemm_strided_batched,
// src/interface/gemm_interface.hpp:200-240, with Gemm's batch loop in
// src/operations/blas3/gemm_local.hpp:438-516); each problem here keeps the
// blas::_gemm semantics (alpha/beta rules, any transposes, column-major).
//
// Scheduler: the problems' 64x64 output tiles are numbered in problem order
// (prefix sums of per-problem tile counts in the device problem table).
// Every CTA of a persistent grid (a multiple of the SM count) takes the next
// tile number from a global atomic counter, finds its problem by binary
// search, and computes the tile; no CTA ever waits on another.  The last CTA
// to finish resets the counters, so the same launch can be replayed from a
// CUDA graph with no host work.
//
// Tile compute: A and B slabs (BK = 16) are converted from FP32 or BF16 to
// FP32 as they are staged in shared memory (any transpose), and each of 256
// threads accumulates a 4x4 FP32 register tile.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "gemm_internal.cuh"
#include "grouped_tc.cuh"

namespace gb {

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
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int gn = n0 + tx * 4 + j;
    if (gn >= p.n) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int gm = m0 + ty * 4 + i;
      if (gm >= p.m) continue;
      float* cp = p.c + gm + int64_t(gn) * p.ldc;
      float v = p.alpha * acc[i][j];
      if (p.beta != 0.f) v = fmaf(p.beta, *cp, v);
      *cp = v;
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

// A grouped plan: the device problem table, the scheduler counters and the
// instantiated CUDA graph of the persistent launch.
struct gbblas_grouped_plan_s {
  int dtype = 0;
  int method = 1;  // 1: tcgen05 tiles (128 x 64), 0: SIMT tiles (64 x 64)
  int count = 0;
  int64_t total_tiles = 0;
  int grid = 0;
  gb::GroupedProblem* table = nullptr;
  unsigned long long* counters = nullptr;
  cudaGraphExec_t exec = nullptr;
  int device = 0;
  int* err = nullptr;  // device error word of the creating handle
};

using namespace gb;

static gbblas_status_t launch_grouped(cudaStream_t s, gbblas_grouped_plan_s* p, int* err) {
  if (p->method == 1) {
    if (p->dtype == GBBLAS_DTYPE_BF16) {
      static bool attr = false;
      if (!attr) {
        GB_CUDA_TRY(cudaFuncSetAttribute(grouped_tc_kernel<__nv_bfloat16, 1, GroupedProblem>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, GtCfg<1>::SMEM));
        attr = true;
      }
      grouped_tc_kernel<__nv_bfloat16, 1, GroupedProblem><<<p->grid, kGtThreads, GtCfg<1>::SMEM, s>>>(
          p->table, p->count, p->total_tiles, p->counters, err);
    } else {
      static bool attr = false;
      if (!attr) {
        GB_CUDA_TRY(cudaFuncSetAttribute(grouped_tc_kernel<float, 3, GroupedProblem>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, GtCfg<3>::SMEM));
        attr = true;
      }
      grouped_tc_kernel<float, 3, GroupedProblem><<<p->grid, kGtThreads, GtCfg<3>::SMEM, s>>>(
          p->table, p->count, p->total_tiles, p->counters, err);
    }
    return after_launch("grouped_tc");
  }
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
  if (plan->table) cudaFree(plan->table);
  if (plan->counters) cudaFree(plan->counters);
  delete plan;
  return GBBLAS_STATUS_SUCCESS;
}

static gbblas_status_t build_table(int dtype, int64_t count, const char* transa, const char* transb,
                                   const int64_t* m, const int64_t* n, const int64_t* k, const float* alpha,
                                   const void* const* a, const int64_t* lda, const void* const* b,
                                   const int64_t* ldb, const float* beta, float* const* c, const int64_t* ldc,
                                   int tile_m, int tile_n, std::vector<GroupedProblem>& tab, int64_t& tiles) {
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
    p.tile_start = tiles;
    p.alpha = alpha[i];
    p.beta = beta[i];
    p.a = a[i];
    p.b = b[i];
    p.c = c[i];
    p.lda = lda[i];
    p.ldb = ldb[i];
    p.ldc = ldc[i];
    tiles += cdiv(m[i], tile_m) * p.tiles_n;
    tab.push_back(p);
  }
  return GBBLAS_STATUS_SUCCESS;
}

static int grouped_grid(gbblas_handle_t h, int64_t tiles, int method, int dtype) {
  // resident CTAs per SM: SIMT 8 x 256 threads; tcgen05 by shared memory
  const int per_sm = method == 0 ? 8 : (dtype == GBBLAS_DTYPE_BF16 ? 2 : 1);
  const int64_t cap = int64_t(h->sm_count) * per_sm;
  return int(std::max<int64_t>(1, std::min<int64_t>(tiles, cap)));
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
  std::vector<GroupedProblem> tab;
  int64_t tiles = 0;
  const int method = grouped_method();
  GB_TRY(build_table(dtype, count, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc,
                     method ? kGtBM : kGT, method ? kGtBN : kGT, tab, tiles));
  auto* plan = new (std::nothrow) gbblas_grouped_plan_s();
  if (!plan) return fail(GBBLAS_STATUS_ALLOC_FAILED, "grouped: out of host memory");
  plan->dtype = dtype;
  plan->method = method;
  plan->err = h->dev_error;
  plan->count = int(tab.size());
  plan->total_tiles = tiles;
  plan->device = h->device;
  plan->grid = grouped_grid(h, tiles, method, dtype);
  cudaError_t e = cudaMalloc(&plan->table, sizeof(GroupedProblem) * std::max<size_t>(1, tab.size()));
  if (e == cudaSuccess) e = cudaMalloc(&plan->counters, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(plan->counters, 0, 2 * sizeof(unsigned long long));
  if (e == cudaSuccess && !tab.empty())
    e = cudaMemcpy(plan->table, tab.data(), sizeof(GroupedProblem) * tab.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    gbblas_grouped_plan_destroy(plan);
    return cuda_fail(e, "grouped: plan upload");
  }
  *out = plan;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_grouped_plan_run(gbblas_handle_t h, gbblas_grouped_plan_t plan) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "grouped: null handle");
  if (!plan) return fail(GBBLAS_STATUS_INVALID_ARG, "grouped: null plan");
  if (plan->total_tiles == 0) return GBBLAS_STATUS_SUCCESS;
  if (!plan->exec) {
    // capture the persistent launch once on a private stream (the handle's
    // stream may be the legacy default stream, which cannot be captured)
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
  std::vector<GroupedProblem> tab;
  int64_t tiles = 0;
  const int method = grouped_method();
  GB_TRY(build_table(dtype, count, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc,
                     method ? kGtBM : kGT, method ? kGtBN : kGT, tab, tiles));
  if (tiles == 0) return GBBLAS_STATUS_SUCCESS;
  // one-shot: table and counters live in the handle's stream-ordered temp memory
  const size_t tbytes = (sizeof(GroupedProblem) * tab.size() + 255) & ~size_t(255);
  void* ws = nullptr;
  GB_TRY(temp_acquire(h, tbytes + 256, &ws));
  gbblas_grouped_plan_s tmp;
  tmp.dtype = dtype;
  tmp.method = method;
  tmp.count = int(tab.size());
  tmp.total_tiles = tiles;
  tmp.grid = grouped_grid(h, tiles, method, dtype);
  tmp.table = static_cast<GroupedProblem*>(ws);
  tmp.counters = reinterpret_cast<unsigned long long*>(static_cast<uint8_t*>(ws) + tbytes);
  GB_CUDA_TRY(cudaMemcpyAsync(tmp.table, tab.data(), sizeof(GroupedProblem) * tab.size(), cudaMemcpyHostToDevice,
                              h->stream));
  GB_CUDA_TRY(cudaMemsetAsync(tmp.counters, 0, 2 * sizeof(unsigned long long), h->stream));
  gbblas_status_t s = launch_grouped(h->stream, &tmp, h->dev_error);
  tmp.table = nullptr;  // not owned
  tmp.counters = nullptr;
  return s;
}

}  // extern "C"

// matvec.cuh — the two HBM-bound column-major matrix sweeps shared by GEMV
// and extension::_reduction.
//
//   rows sweep  (GEMV 'n', reduction outer): out(i) = fold_j  f(A(i,j), x_j)
//   cols sweep  (GEMV 't', reduction inner): out(j) = fold_i  f(A(i,j), x_i)
//
// Both read A exactly once with 128-bit coalesced loads (when lda and the
// base allow it), keep several loads in flight per thread, and split the
// folded dimension across CTAs when the preserved dimension alone cannot
// fill the 152 SMs.  Split partials go to temp memory; the last CTA of each
// output tile (a per-tile ticket, no waiting) folds them in split order and
// runs the epilogue, so results are deterministic.
//
// Policy supplies: Acc, init(), add(acc, a, x), merge(acc, other),
// finish(acc, out_index) -> writes the output element.
#pragma once

#include "common.cuh"
#include "reduce_util.cuh"

namespace gb {

template <typename T>
struct Pack16;
template <>
struct Pack16<float> {
  using V = float4;
  static constexpr int n = 4;
  __device__ static void get(const V& v, float* o) { o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w; }
};
template <>
struct Pack16<double> {
  using V = double2;
  static constexpr int n = 2;
  __device__ static void get(const V& v, double* o) { o[0] = v.x; o[1] = v.y; }
};

constexpr int kMvThreads = 256;
constexpr int kMvWarps = kMvThreads / 32;

// ------------------------------------------------------- warp per column --
// out(j) = fold over i of pol.add(A[i + j*lda], x[i]) with one warp per
// column j: lane l reads the 16-byte vectors l, l + 32, ... of the column
// (kCwUnroll in flight) and, with HAS_X, the matching x through L1, then a
// fixed shuffle tree; no partial sums, no fold across CTAs, the same order on
// every run.  The grid is at most one wave (kCwCtas CTAs of 8 warps per SM,
// 64 registers) and column j goes to warp j / grid of CTA j % grid, so the
// CTAs get the same number of columns to within one.  ALIGNED: the columns
// (and x) are 16-byte aligned; otherwise each column's elements before its
// first 16-byte boundary are read one per lane, the rest as 16-byte vectors,
// and x one element per lane, so a leading dimension TMA cannot address
// keeps the vector loads of A.
constexpr int kCwUnroll = 4, kCwCtas = 4;

template <class P, typename T, bool HAS_X, bool ALIGNED>
__global__ void __launch_bounds__(kMvThreads, kCwCtas)
    cols_warp(P pol, int64_t m, int64_t n, const T* __restrict__ A, int64_t lda, const T* __restrict__ x) {
  using V = typename Pack16<T>::V;
  using Acc = typename P::Acc;
  constexpr int W = Pack16<T>::n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t step = int64_t(kMvWarps) * gridDim.x;
  const int64_t first = int64_t(warp) * gridDim.x + blockIdx.x;
  for (int64_t j = first; j < n; j += step) {
    const T* col = A + j * lda;
    Acc acc = pol.init();
    int64_t head = 0;  // elements before the column's first 16-byte boundary
    if (!ALIGNED) {
      head = int64_t(((16 - (reinterpret_cast<uintptr_t>(col) & 15)) & 15) / sizeof(T));
      if (head > m) head = m;
      if (lane < head) pol.add(acc, col[lane], HAS_X ? x[lane] : T(1));
    }
    const V* av = reinterpret_cast<const V*>(col + head);
    const T* xh = HAS_X ? x + head : x;
    const int64_t nv = (m - head) / W;  // whole vectors after the head
    int64_t v = lane;
    for (; v + 32 * (kCwUnroll - 1) < nv; v += 32 * kCwUnroll) {
      V a[kCwUnroll];
#pragma unroll
      for (int u = 0; u < kCwUnroll; ++u) a[u] = __ldcs(av + v + 32 * u);
      if (HAS_X && ALIGNED) {
        V b[kCwUnroll];
#pragma unroll
        for (int u = 0; u < kCwUnroll; ++u) b[u] = __ldg(reinterpret_cast<const V*>(xh) + v + 32 * u);
#pragma unroll
        for (int u = 0; u < kCwUnroll; ++u) {
          T ae[W], be[W];
          Pack16<T>::get(a[u], ae);
          Pack16<T>::get(b[u], be);
#pragma unroll
          for (int e = 0; e < W; ++e) pol.add(acc, ae[e], be[e]);
        }
      } else {
#pragma unroll
        for (int u = 0; u < kCwUnroll; ++u) {
          T ae[W];
          Pack16<T>::get(a[u], ae);
#pragma unroll
          for (int e = 0; e < W; ++e) pol.add(acc, ae[e], HAS_X ? __ldg(xh + (v + 32 * u) * W + e) : T(1));
        }
      }
    }
    for (; v < nv; v += 32) {
      T ae[W];
      Pack16<T>::get(__ldcs(av + v), ae);
#pragma unroll
      for (int e = 0; e < W; ++e) pol.add(acc, ae[e], HAS_X ? __ldg(xh + v * W + e) : T(1));
    }
    for (int64_t i = head + nv * W + lane; i < m; i += 32) pol.add(acc, col[i], HAS_X ? x[i] : T(1));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const Acc o = pol.shfl_down(acc, off);
      pol.merge(acc, o);
    }
    if (lane == 0) pol.finish(acc, j);
  }
}

// ----------------------------------------------- CTA per column group --
// out(j) = fold over i of pol.add(A[i + j*lda], x[i]) for 16-byte-aligned
// columns and x: CTA b takes columns b, b + grid, ... (the CTAs' counts
// differ by at most one) and, for each, its eight warps take equal
// contiguous row ranges (whole 32-vector rounds), so every warp of the wave
// streams the same number of bytes; each warp folds its range with a fixed
// shuffle tree and the CTA's thread t folds column t's eight warp partials
// in warp order (deterministic).  One warp per column leaves the wave
// uneven when the columns are not a whole number per warp (8192 columns on
// 4864 warps: 1536 warps with one column, 3328 with two).
constexpr int kCcMaxCols = 16;
static_assert(2 * kMvWarps <= kCcMaxCols && kCcMaxCols <= kMvThreads, "cols_cta column budget");

template <class P, typename T>
__global__ void __launch_bounds__(kMvThreads, kCwCtas)
    cols_cta(P pol, int64_t m, int64_t n, const T* __restrict__ A, int64_t lda, const T* __restrict__ x) {
  using V = typename Pack16<T>::V;
  using Acc = typename P::Acc;
  constexpr int W = Pack16<T>::n;
  __shared__ Acc red[kCcMaxCols][kMvWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nv = m / W;  // whole vectors per column; the last warp adds the m % W tail rows
  const int64_t per = (((nv + kMvWarps - 1) / kMvWarps) + 31) / 32 * 32;
  const int64_t v0 = int64_t(warp) * per, v1 = v0 + per < nv ? v0 + per : nv;
  const V* xv = reinterpret_cast<const V*>(x);
  int cols = 0;
  for (int64_t j = blockIdx.x; j < n && cols < kCcMaxCols; j += gridDim.x, ++cols) {
    const V* av = reinterpret_cast<const V*>(A + j * lda);
    Acc acc = pol.init();
    int64_t v = v0 + lane;
    for (; v + 32 * (kCwUnroll - 1) < v1; v += 32 * kCwUnroll) {
      V a[kCwUnroll], b[kCwUnroll];
#pragma unroll
      for (int u = 0; u < kCwUnroll; ++u) a[u] = __ldcs(av + v + 32 * u);
#pragma unroll
      for (int u = 0; u < kCwUnroll; ++u) b[u] = __ldg(xv + v + 32 * u);
#pragma unroll
      for (int u = 0; u < kCwUnroll; ++u) {
        T ae[W], be[W];
        Pack16<T>::get(a[u], ae);
        Pack16<T>::get(b[u], be);
#pragma unroll
        for (int e = 0; e < W; ++e) pol.add(acc, ae[e], be[e]);
      }
    }
    for (; v < v1; v += 32) {
      T ae[W], be[W];
      Pack16<T>::get(__ldcs(av + v), ae);
      Pack16<T>::get(__ldg(xv + v), be);
#pragma unroll
      for (int e = 0; e < W; ++e) pol.add(acc, ae[e], be[e]);
    }
    if (warp == kMvWarps - 1 && lane < m - nv * W) {
      const T* col = A + j * lda;
      pol.add(acc, col[nv * W + lane], x[nv * W + lane]);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const Acc o = pol.shfl_down(acc, off);
      pol.merge(acc, o);
    }
    if (lane == 0) red[cols][warp] = acc;
  }
  __syncthreads();
  if (int(threadIdx.x) < cols) {
    Acc acc = red[threadIdx.x][0];
#pragma unroll
    for (int w = 1; w < kMvWarps; ++w) pol.merge(acc, red[threadIdx.x][w]);
    pol.finish(acc, int64_t(blockIdx.x) + int64_t(threadIdx.x) * gridDim.x);
  }
}

// Launches cols_cta (16-byte-aligned columns and x) or cols_warp when one
// applies and returns true (status in *st): x contiguous (or no x), at least
// a quarter column per warp of the wave, and either aligned columns and x
// with at most two columns per warp (when aligned_ok), or columns TMA cannot
// address at any width.
template <class P, typename T, bool HAS_X>
inline bool try_cols_warp(gbblas_handle_t h, const P& pol, int64_t m, int64_t n, const T* A, int64_t lda,
                          const T* x, bool aligned_ok, gbblas_status_t* st) {
  constexpr int W = 16 / int(sizeof(T));
  const int64_t slots = int64_t(kCwCtas) * h->sm_count, warps = slots * kMvWarps;
  if (m <= 0 || 4 * n < warps) return false;
  const int64_t want = (n + kMvWarps - 1) / kMvWarps;
  const unsigned grid = unsigned(want < slots ? want : slots);
  const bool vec_a = lda % W == 0 && aligned16(A);
  if (vec_a && (!HAS_X || aligned16(x))) {
    if (!aligned_ok || n > 2 * warps) return false;
    if (HAS_X) {
      // at most 2 * kMvWarps <= kCcMaxCols columns per CTA
      const unsigned cgrid = unsigned(n < slots ? n : slots);
      cols_cta<P, T><<<cgrid, kMvThreads, 0, h->stream>>>(pol, m, n, A, lda, x);
    } else {
      cols_warp<P, T, HAS_X, true><<<grid, kMvThreads, 0, h->stream>>>(pol, m, n, A, lda, x);
    }
  } else if (!vec_a) {
    cols_warp<P, T, HAS_X, false><<<grid, kMvThreads, 0, h->stream>>>(pol, m, n, A, lda, x);
  } else {
    return false;  // aligned columns with an unaligned x: the TMA sweep
  }
  *st = after_launch("cols_warp");
  return true;
}

// ------------------------------------------------------------- rows sweep --
// CTA = 8 warps over a block of 32*RPT rows; warp w takes columns
// c0+w, c0+w+8, ... of its split; the 8 warp partials fold in warp order.
// VEC: lane l owns rows RPT*l .. RPT*l + RPT-1 (one 16-byte load per
// column); otherwise rows l, l + 32, ..., so each element-wise load of a
// warp covers 32 consecutive rows (one 128-byte line instead of a 512-byte
// span at a 16-byte stride).
template <class P, typename T, bool VEC, bool HAS_X>
__global__ void __launch_bounds__(kMvThreads, 4)
    rows_sweep(P pol, int64_t M, int64_t N, const T* __restrict__ A, int64_t lda, const T* __restrict__ xb,
               int64_t incx, int64_t cols_per_split, typename P::Acc* __restrict__ partials,
               unsigned int* __restrict__ tickets) {
  using Acc = typename P::Acc;
  constexpr int RPT = Pack16<T>::n;
  constexpr int WR = 32 * RPT;
  __shared__ Acc red[kMvWarps][WR];
  __shared__ bool is_last;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t rblock = blockIdx.x;
  // offset (within the block) of the r-th row this lane owns
  auto rof = [&](int r) { return VEC ? lane * RPT + r : r * 32 + lane; };
  const int64_t row0 = rblock * WR + rof(0);
  const int64_t c0 = int64_t(blockIdx.y) * cols_per_split;
  const int64_t c1 = min(N, c0 + cols_per_split);
  Acc acc[RPT];
#pragma unroll
  for (int r = 0; r < RPT; ++r) acc[r] = pol.init();
  const bool full = VEC && (row0 + RPT <= M);
  const T* Ab = A + rblock * WR;

  auto load_col = [&](int64_t j, T* v) {
    if (full) {
      Pack16<T>::get(__ldcs(reinterpret_cast<const typename Pack16<T>::V*>(Ab + rof(0) + j * lda)), v);
    } else {
#pragma unroll
      for (int r = 0; r < RPT; ++r) v[r] = (rblock * WR + rof(r) < M) ? Ab[j * lda + rof(r)] : T(0);
    }
  };

  int64_t j = c0 + warp;
  constexpr int U = 4;
  for (; j + (U - 1) * kMvWarps < c1; j += U * kMvWarps) {
    T v[U][RPT];
    T xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      load_col(j + u * kMvWarps, v[u]);
      xv[u] = HAS_X ? xb[(j + u * kMvWarps) * incx] : T(1);
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int r = 0; r < RPT; ++r) pol.add(acc[r], v[u][r], xv[u]);
  }
  for (; j < c1; j += kMvWarps) {
    T v[RPT];
    load_col(j, v);
    T xv = HAS_X ? xb[j * incx] : T(1);
#pragma unroll
    for (int r = 0; r < RPT; ++r) pol.add(acc[r], v[r], xv);
  }
#pragma unroll
  for (int r = 0; r < RPT; ++r) red[warp][rof(r)] = acc[r];
  __syncthreads();
  const int t = threadIdx.x;
  const int64_t row = rblock * WR + t;
  Acc s;
  if (t < WR) {
    s = red[0][t];
#pragma unroll
    for (int w = 1; w < kMvWarps; ++w) pol.merge(s, red[w][t]);
  }
  if (gridDim.y == 1) {
    if (t < WR && row < M) pol.finish(s, row);
    return;
  }
  if (t < WR && row < M) partials[int64_t(blockIdx.y) * M + row] = s;
  __threadfence();
  __syncthreads();
  if (t == 0) is_last = atomicAdd(tickets + rblock, 1u) == gridDim.y - 1;
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (t < WR && row < M) {
    Acc f = ldcg_any(partials + row);
    for (unsigned sp = 1; sp < gridDim.y; ++sp) pol.merge(f, ldcg_any(partials + int64_t(sp) * M + row));
    pol.finish(f, row);
  }
  if (t == 0) tickets[rblock] = 0u;
}

// ------------------------------------------------------------ narrow rows --
// Matrices of at most kNarrowRows rows (short and wide).  One warp-wide
// load of the sweeps above covers 32 x (16 / sizeof(T)) rows of ONE column,
// so with 8 rows a warp read 32 useful bytes per load and GEMV 'n' 8 x 2^22
// ran at 356 GB/s.  Here a column takes `lpc` lanes (rows / RPT rounded up to
// a power of two) and a warp covers 32 / lpc columns per load: a packed A
// (lda == rows) streams in contiguous 512-byte warp loads.
constexpr int kNarrowRows = 128;  // FP32 (32 lanes x 4 rows); FP64: 64
template <typename T>
constexpr int narrow_rows() {
  return 32 * (16 / int(sizeof(T)));
}
constexpr int kThreadRows = 32;  // GEMV 't': one thread per column up to here, cols_lanes above

// out(i) = fold over j of pol.add(A[i + j*lda], x[j]), i < M <= narrow_rows<T>().
// CTA b takes columns [b*cols_per_cta, ...); lanes with the same row group
// are folded by shuffles, warps in warp order in shared memory, and the
// CTAs' per-row partials by the last CTA to finish, all 256 threads over
// equal runs of CTAs, then the runs in order.
template <class P, typename T, bool VEC, bool HAS_X>
__global__ void __launch_bounds__(kMvThreads)
    rows_narrow(P pol, int M, int64_t N, const T* __restrict__ A, int64_t lda, const T* __restrict__ xb,
                int64_t incx, int lpc_log2, int64_t cols_per_cta, typename P::Acc* __restrict__ partials,
                unsigned int* __restrict__ tickets) {
  using Acc = typename P::Acc;
  constexpr int RPT = Pack16<T>::n;
  __shared__ Acc red[kMvWarps * kNarrowRows];  // [warp][row], later [run][row]
  __shared__ bool is_last;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lpc = 1 << lpc_log2, cpw = 32 >> lpc_log2;
  const int r0 = (lane & (lpc - 1)) * RPT;
  const int64_t c0 = int64_t(blockIdx.x) * cols_per_cta;
  const int64_t c1 = min(N, c0 + cols_per_cta);
  const int64_t step = int64_t(cpw) * kMvWarps;
  const bool full = VEC && r0 + RPT <= M;
  Acc acc[RPT];
#pragma unroll
  for (int r = 0; r < RPT; ++r) acc[r] = pol.init();
  auto load_col = [&](int64_t j, T* v) {
    const T* col = A + j * lda + r0;
    if (full) {
      Pack16<T>::get(__ldcs(reinterpret_cast<const typename Pack16<T>::V*>(col)), v);
    } else {
#pragma unroll
      for (int r = 0; r < RPT; ++r) v[r] = r0 + r < M ? col[r] : T(0);
    }
  };
  int64_t j = c0 + warp * cpw + (lane >> lpc_log2);
  constexpr int U = 4;
  for (; j + (U - 1) * step < c1; j += U * step) {
    T v[U][RPT];
    T xv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      load_col(j + u * step, v[u]);
      xv[u] = HAS_X ? xb[(j + u * step) * incx] : T(1);
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int r = 0; r < RPT; ++r) pol.add(acc[r], v[u][r], xv[u]);
  }
  for (; j < c1; j += step) {
    T v[RPT];
    load_col(j, v);
    const T xv = HAS_X ? xb[j * incx] : T(1);
#pragma unroll
    for (int r = 0; r < RPT; ++r) pol.add(acc[r], v[r], xv);
  }
  // lanes l, l + lpc, l + 2 lpc, ... hold the same rows: fold them into lane l
  for (int off = 16; off >= lpc; off >>= 1)
#pragma unroll
    for (int r = 0; r < RPT; ++r) pol.merge(acc[r], pol.shfl_down(acc[r], off));
  if (lane < lpc)
#pragma unroll
    for (int r = 0; r < RPT; ++r) red[warp * kNarrowRows + r0 + r] = acc[r];
  __syncthreads();
  const int t = threadIdx.x;
  Acc s;
  if (t < M) {
    s = red[t];
    for (int w = 1; w < kMvWarps; ++w) pol.merge(s, red[w * kNarrowRows + t]);
  }
  if (gridDim.x == 1) {
    if (t < M) pol.finish(s, t);
    return;
  }
  if (t < M) partials[int64_t(blockIdx.x) * M + t] = s;
  __threadfence();
  __syncthreads();
  if (t == 0) is_last = atomicAdd(tickets, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  const int runs = kMvThreads / M;
  const int64_t per = (int64_t(gridDim.x) + runs - 1) / runs;
  if (t < runs * M) {
    const int row = t % M, run = t / M;
    const int64_t b0 = run * per, b1 = min(int64_t(gridDim.x), b0 + per);
    Acc f = pol.init();
    for (int64_t b = b0; b < b1; ++b) pol.merge(f, ldcg_any(partials + b * M + row));
    red[run * M + row] = f;
  }
  __syncthreads();
  if (t < M) {
    Acc f = red[t];
    for (int run = 1; run < runs; ++run) pol.merge(f, red[run * M + t]);
    pol.finish(f, t);
  }
  if (t == 0) tickets[0] = 0u;
}

// out(j) = fold over i < M of pol.add(A[i + j*lda], x[i]), M <= kThreadRows (32):
// one thread per column, its M values in at most 8 (FP32) 16-byte loads; x
// in shared memory.  A packed A streams as contiguous 1 KB warp loads (8 x
// 2^22 GEMV 't' ran at 221 GB/s with a warp per column).
template <class P, typename T, bool VEC, bool HAS_X>
__global__ void __launch_bounds__(kMvThreads)
    cols_thread(P pol, int M, int64_t N, const T* __restrict__ A, int64_t lda, const T* __restrict__ xb,
                int64_t incx) {
  using Acc = typename P::Acc;
  constexpr int RPT = Pack16<T>::n;
  __shared__ T xs[kThreadRows];
  if (threadIdx.x < M) xs[threadIdx.x] = HAS_X ? xb[int64_t(threadIdx.x) * incx] : T(1);
  __syncthreads();
  const int64_t j = int64_t(blockIdx.x) * kMvThreads + threadIdx.x;
  if (j >= N) return;
  const T* col = A + j * lda;
  Acc acc = pol.init();
  if (VEC) {
    int i = 0;
    for (; i + RPT <= M; i += RPT) {
      T v[RPT];
      Pack16<T>::get(__ldcs(reinterpret_cast<const typename Pack16<T>::V*>(col + i)), v);
#pragma unroll
      for (int r = 0; r < RPT; ++r) pol.add(acc, v[r], xs[i + r]);
    }
    for (; i < M; ++i) pol.add(acc, col[i], xs[i]);
  } else {
    for (int i = 0; i < M; ++i) pol.add(acc, col[i], xs[i]);
  }
  pol.finish(acc, j);
}

// out(j) = fold over i < M of pol.add(A[i + j*lda], x[i]), kThreadRows < M <= narrow_rows<T>():
// a column takes `lpc` lanes as in rows_narrow, each lane one 16-byte group
// of its rows (x of those rows held in registers), folded by shuffles in a
// fixed tree; a warp covers 32 / lpc columns per load, so a packed A streams
// in contiguous 512-byte warp loads (8 x 2^22 GEMV 't' ran at 221 GB/s with
// a warp per column).  Grid-stride over columns, warp-uniform, so that every
// lane takes part in the shuffles.
template <class P, typename T, bool VEC, bool HAS_X>
__global__ void __launch_bounds__(kMvThreads)
    cols_lanes(P pol, int M, int64_t N, const T* __restrict__ A, int64_t lda, const T* __restrict__ xb,
               int64_t incx, int lpc_log2) {
  using Acc = typename P::Acc;
  constexpr int RPT = Pack16<T>::n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lpc = 1 << lpc_log2, cpw = 32 >> lpc_log2;
  const int sub = lane & (lpc - 1), r0 = sub * RPT;
  T xr[RPT];
#pragma unroll
  for (int r = 0; r < RPT; ++r) xr[r] = r0 + r < M ? (HAS_X ? xb[int64_t(r0 + r) * incx] : T(1)) : T(0);
  const bool full = VEC && r0 + RPT <= M;
  const int64_t step = int64_t(cpw) * kMvWarps * gridDim.x;
  constexpr int U = 4;
  for (int64_t base = (int64_t(blockIdx.x) * kMvWarps + warp) * cpw; base < N; base += U * step) {
    Acc acc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      // columns past N read column N - 1 (in bounds, unconditional, so the U
      // loads issue together) and are not stored
      int64_t j = base + u * step + (lane >> lpc_log2);
      if (j >= N) j = N - 1;
      const T* col = A + j * lda + r0;
      T v[RPT];
      if (full) {
        Pack16<T>::get(__ldcs(reinterpret_cast<const typename Pack16<T>::V*>(col)), v);
      } else {
#pragma unroll
        for (int r = 0; r < RPT; ++r) v[r] = r0 + r < M ? col[r] : T(0);
      }
      acc[u] = pol.init();
#pragma unroll
      for (int r = 0; r < RPT; ++r) pol.add(acc[u], v[r], xr[r]);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      for (int off = lpc >> 1; off > 0; off >>= 1) pol.merge(acc[u], pol.shfl_down(acc[u], off));
      const int64_t j = base + u * step + (lane >> lpc_log2);
      if (sub == 0 && j < N) pol.finish(acc[u], j);
    }
  }
}

// out(i) = fold over j < N of pol.add(A[i + j*lda], x[j]) for tall, narrow A
// (N <= kTallCols): a warp owns 32 x RPT rows over every column, so a lane
// keeps N loads of its rows in flight and no partial sums cross warps (the
// rows sweep gave each warp one column of 128 rows: 4M x 8 GEMV 'n' at
// 2207 GB/s).
constexpr int kTallCols = 32;

template <class P, typename T, bool VEC, bool HAS_X>
__global__ void __launch_bounds__(kMvThreads)
    rows_tall(P pol, int64_t M, int N, const T* __restrict__ A, int64_t lda, const T* __restrict__ xb,
              int64_t incx) {
  using Acc = typename P::Acc;
  constexpr int RPT = Pack16<T>::n;
  constexpr int WR = 32 * RPT;
  __shared__ T xs[kTallCols];
  if (threadIdx.x < N) xs[threadIdx.x] = HAS_X ? xb[int64_t(threadIdx.x) * incx] : T(1);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t rb = (int64_t(blockIdx.x) * kMvWarps + warp) * WR;
  if (rb >= M) return;
  // offset (within the warp's rows) of the r-th row this lane owns
  auto rof = [&](int r) { return VEC ? lane * RPT + r : r * 32 + lane; };
  const bool full = VEC && rb + rof(0) + RPT <= M;
  const T* Ab = A + rb;
  Acc acc[RPT];
#pragma unroll
  for (int r = 0; r < RPT; ++r) acc[r] = pol.init();
  constexpr int U = 8;
  int j = 0;
  for (; j + U <= N; j += U) {
    T v[U][RPT];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const T* col = Ab + int64_t(j + u) * lda;
      if (full) {
        Pack16<T>::get(__ldcs(reinterpret_cast<const typename Pack16<T>::V*>(col + rof(0))), v[u]);
      } else {
#pragma unroll
        for (int r = 0; r < RPT; ++r) v[u][r] = rb + rof(r) < M ? col[rof(r)] : T(0);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int r = 0; r < RPT; ++r) pol.add(acc[r], v[u][r], xs[j + u]);
  }
  for (; j < N; ++j) {
    const T* col = Ab + int64_t(j) * lda;
    T v[RPT];
    if (full) {
      Pack16<T>::get(__ldcs(reinterpret_cast<const typename Pack16<T>::V*>(col + rof(0))), v);
    } else {
#pragma unroll
      for (int r = 0; r < RPT; ++r) v[r] = rb + rof(r) < M ? col[rof(r)] : T(0);
    }
#pragma unroll
    for (int r = 0; r < RPT; ++r) pol.add(acc[r], v[r], xs[j]);
  }
#pragma unroll
  for (int r = 0; r < RPT; ++r)
    if (rb + rof(r) < M) pol.finish(acc[r], rb + rof(r));
}

// ------------------------------------------------------------- cols sweep --
// CTA = 8 warps over CC columns and one chunk of `rows_per_split` rows; x of
// the chunk is staged in shared memory; warp w takes columns w, w+8, ... and
// reads each column chunk with 128-bit loads, 4 in flight per lane.
template <class P, typename T, bool VEC, bool HAS_X>
__global__ void __launch_bounds__(kMvThreads, 8)
    cols_sweep(P pol, int64_t M, int64_t N, const T* __restrict__ A, int64_t lda, const T* __restrict__ xb,
               int64_t incx, int64_t rows_per_split, int cols_per_cta, typename P::Acc* __restrict__ partials,
               unsigned int* __restrict__ tickets) {
  using Acc = typename P::Acc;
  constexpr int RPT = Pack16<T>::n;
  constexpr int WR = 32 * RPT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* xs = reinterpret_cast<T*>(smem_raw);
  Acc* colres = reinterpret_cast<Acc*>(smem_raw + ((rows_per_split * sizeof(T) + 15) & ~size_t(15)));
  __shared__ bool is_last;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t r0 = int64_t(blockIdx.y) * rows_per_split;
  const int64_t rlen = min(M - r0, rows_per_split);
  if (HAS_X)
    for (int64_t t = threadIdx.x; t < rows_per_split; t += blockDim.x) xs[t] = t < rlen ? xb[(r0 + t) * incx] : T(0);
  __syncthreads();
  const int64_t cbase = int64_t(blockIdx.x) * cols_per_cta;
  for (int cc = warp; cc < cols_per_cta; cc += kMvWarps) {
    const int64_t jcol = cbase + cc;
    if (jcol >= N) break;
    const T* col = A + jcol * lda + r0;
    constexpr int U = 4;
    Acc acc[U];
#pragma unroll
    for (int u = 0; u < U; ++u) acc[u] = pol.init();
    int64_t r = int64_t(lane) * RPT;
    if (VEC) {
      for (; r + (U - 1) * WR + RPT <= rlen; r += U * WR) {
        T v[U][RPT];
#pragma unroll
        for (int u = 0; u < U; ++u)
          Pack16<T>::get(__ldcs(reinterpret_cast<const typename Pack16<T>::V*>(col + r + u * WR)), v[u]);
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int e = 0; e < RPT; ++e) pol.add(acc[u], v[u][e], HAS_X ? xs[r + u * WR + e] : T(1));
      }
    }
    for (; r < rlen; r += WR) {
#pragma unroll
      for (int e = 0; e < RPT; ++e)
        if (r + e < rlen) pol.add(acc[0], col[r + e], HAS_X ? xs[r + e] : T(1));
    }
#pragma unroll
    for (int u = 1; u < U; ++u) pol.merge(acc[0], acc[u]);
    Acc s = acc[0];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) pol.merge(s, pol.shfl_down(s, off));
    if (lane == 0) {
      if (gridDim.y == 1) pol.finish(s, jcol);
      else colres[cc] = s;
    }
  }
  if (gridDim.y == 1) return;
  __syncthreads();
  for (int cc = threadIdx.x; cc < cols_per_cta; cc += blockDim.x) {
    const int64_t jcol = cbase + cc;
    if (jcol < N) partials[int64_t(blockIdx.y) * N + jcol] = colres[cc];
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = atomicAdd(tickets + blockIdx.x, 1u) == gridDim.y - 1;
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  // every thread folds a run of the splits for one column, then the runs are
  // folded in order (a long, narrow A has over a thousand splits; folded by
  // one thread per column they dominated 4M x 8 GEMV 't')
  __shared__ Acc runsum[kMvThreads];
  const int runs = kMvThreads / cols_per_cta;
  const int64_t nsp = gridDim.y, per = (nsp + runs - 1) / runs;
  {
    const int cc = threadIdx.x % cols_per_cta, run = threadIdx.x / cols_per_cta;
    if (run < runs) {
      Acc f = pol.init();
      const int64_t s1 = min(nsp, (run + 1) * per);
      if (cbase + cc < N)
        for (int64_t sp = run * per; sp < s1; ++sp) pol.merge(f, ldcg_any(partials + sp * N + cbase + cc));
      runsum[run * cols_per_cta + cc] = f;
    }
  }
  __syncthreads();
  for (int cc = threadIdx.x; cc < cols_per_cta; cc += blockDim.x) {
    const int64_t jcol = cbase + cc;
    if (jcol >= N) break;
    Acc f = runsum[cc];
    for (int run = 1; run < runs; ++run) pol.merge(f, runsum[run * cols_per_cta + cc]);
    pol.finish(f, jcol);
  }
  if (threadIdx.x == 0) tickets[blockIdx.x] = 0u;
}

// ------------------------------------------------------------------- host --
struct SweepPlan {
  int64_t split;      // number of CTAs along the folded dimension
  int64_t per_split;  // folded elements per split
  int cols_per_cta;   // cols sweep only
  int64_t tiles;      // CTAs along the preserved dimension
};

// rows sweep: preserved = M (rows), folded = N (cols)
inline SweepPlan plan_rows(int64_t M, int64_t N, int sm_count, int elem_bytes) {
  const int64_t WR = 32 * (16 / elem_bytes);
  SweepPlan p;
  p.tiles = cdiv(M > 0 ? M : 1, WR);
  const int64_t target = int64_t(sm_count) * 4;  // one wave of rows_sweep (4 CTAs per SM)
  int64_t split = cdiv(target, p.tiles);
  const int64_t max_split = cdiv(N > 0 ? N : 1, 64);
  if (split > max_split) split = max_split;
  if (split < 1) split = 1;
  if (p.tiles > int64_t(kMaxTickets)) split = 1;
  p.per_split = split > 1 ? cdiv(N, split) : N;
  p.split = split > 1 ? cdiv(N, p.per_split) : 1;
  p.cols_per_cta = 0;
  return p;
}

// cols sweep: preserved = N (cols), folded = M (rows)
inline SweepPlan plan_cols(int64_t M, int64_t N, int sm_count, int elem_bytes) {
  const int64_t WR = 32 * (16 / elem_bytes);
  SweepPlan p;
  p.cols_per_cta = 32;
  if (N < 8 * int64_t(sm_count)) p.cols_per_cta = 8;
  p.tiles = cdiv(N > 0 ? N : 1, p.cols_per_cta);
  const int64_t target = int64_t(sm_count) * 8;
  int64_t split = cdiv(target, p.tiles);
  const int64_t max_rows = 4096;  // shared-memory x chunk bound
  const int64_t min_split = cdiv(M > 0 ? M : 1, max_rows);
  const int64_t max_split = cdiv(M > 0 ? M : 1, 4 * WR);
  if (split > max_split) split = max_split;
  if (split < min_split) split = min_split;
  if (split < 1) split = 1;
  int64_t per = cdiv(M > 0 ? M : 1, split);
  per = cdiv(per, WR) * WR;
  p.per_split = per;
  p.split = cdiv(M > 0 ? M : 1, per);
  return p;
}

}  // namespace gb

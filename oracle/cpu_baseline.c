/* cpu_baseline.c — the reference's CPU path restated for timing (TEST AND
 * BENCHMARK INFRASTRUCTURE ONLY: only the CPU-baseline leg of bench.py runs
 * these; the product never calls them).
 *
 * portBLAS cannot be built here (no SYCL compiler), so its CPU numbers come
 * from the CBLAS its tests link (OpenBLAS) where CBLAS has the routine and,
 * where it has none or OpenBLAS runs it on one thread, from these OpenMP
 * restatements of portBLAS's own kernels, in FP32 as portBLAS computes them:
 *
 *  - cpu_reduction_f32: extension::_reduction, the Reduction kernel
 *    (src/operations/extension/reduction.hpp:117-230).  Each output keeps
 *    kLanes partial accumulators, lane j summing the reduced elements j,
 *    j + kLanes, ... in FP32 (the reference's per-thread strided loop,
 *    reduction.hpp:137-145), combined by a halving tree (its local-memory
 *    tree, reduction.hpp:205-219).  "inner" reduces each column (contiguous)
 *    to one value; "outer" reduces each row and walks the matrix a block of
 *    rows at a time, column after column, so every read is a contiguous run.
 *  - cpu_iamax_f32: _iamax/_iamin (IndexMaxMin, src/operations/blas1/
 *    IndexMaxMin.hpp with the tuple rule of blas_operators.hpp:276-316): the
 *    first index of the largest (smallest) |x|; each thread scans a
 *    contiguous range, the ranges are combined in order so the first index
 *    wins ties.  OpenBLAS's isamax/isamin run on one thread.
 *
 * Built into liboracle.so with oracle.c (gcc -O2 -fopenmp). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { kLanes = 16, kRowBlock = 512 };

static float tree_sum(float *v, int n) {
  for (int off = n >> 1; off > 0; off >>= 1)
    for (int j = 0; j < off; ++j) v[j] += v[j + off];
  return v[0];
}

/* Add reduction (operator AddOperator; the only one the baseline times).
 * dim 0 = inner (one output per column), 1 = outer (one output per row).
 * Returns 0, or -1 for an operator other than add. */
int cpu_reduction_f32(int op, int dim, const float *in, int64_t ld, int64_t rows, int64_t cols, float *out) {
  if (op != 0) return -1;
  if (dim == 0) {
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < cols; ++c) {
      const float *col = in + c * ld;
      float acc[kLanes] = {0};
      int64_t r = 0;
      for (; r + kLanes <= rows; r += kLanes) {
#pragma omp simd
        for (int j = 0; j < kLanes; ++j) acc[j] += col[r + j];
      }
      for (int j = 0; r + j < rows; ++j) acc[j] += col[r + j];
      out[c] = tree_sum(acc, kLanes);
    }
    return 0;
  }
  const int64_t nblk = (rows + kRowBlock - 1) / kRowBlock;
#pragma omp parallel for schedule(static)
  for (int64_t b = 0; b < nblk; ++b) {
    const int64_t r0 = b * kRowBlock;
    const int64_t nr = rows - r0 < kRowBlock ? rows - r0 : kRowBlock;
    /* acc[lane][row]: lane j sums columns j, j + 4, ... of this row block */
    float acc[4][kRowBlock];
    for (int j = 0; j < 4; ++j)
      for (int64_t i = 0; i < nr; ++i) acc[j][i] = 0.f;
    for (int64_t c = 0; c < cols; ++c) {
      const float *src = in + r0 + c * ld;
      float *a = acc[c & 3];
#pragma omp simd
      for (int64_t i = 0; i < nr; ++i) a[i] += src[i];
    }
    for (int64_t i = 0; i < nr; ++i) out[r0 + i] = (acc[0][i] + acc[2][i]) + (acc[1][i] + acc[3][i]);
  }
  return 0;
}

/* First index of max |x| (is_min = 0) or min |x| (is_min = 1), unit stride.
 * n <= 0 returns 0, as portBLAS's IndexMax of an empty range. */
int64_t cpu_iamax_f32(int64_t n, const float *x, int is_min) {
  if (n <= 0) return 0;
  enum { kMaxThreads = 1024 };
  int64_t best_i[kMaxThreads];
  float best_v[kMaxThreads];
  int nt = 1;
#pragma omp parallel
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#pragma omp single
    nt = omp_get_num_threads() < kMaxThreads ? omp_get_num_threads() : kMaxThreads;
#endif
    if (t < nt) {
      const int64_t chunk = (n + nt - 1) / nt;
      const int64_t lo = (int64_t)t * chunk, hi = lo + chunk < n ? lo + chunk : n;
      int64_t bi = -1;
      float bv = 0.f;
      for (int64_t i = lo; i < hi; ++i) {
        const float a = fabsf(x[i]);
        if (bi < 0 || (is_min ? a < bv : a > bv)) {
          bv = a;
          bi = i;
        }
      }
      best_i[t] = bi;
      best_v[t] = bv;
    }
  }
  int64_t bi = -1;
  float bv = 0.f;
  for (int t = 0; t < nt; ++t) {
    if (best_i[t] < 0) continue;
    if (bi < 0 || (is_min ? best_v[t] < bv : best_v[t] > bv)) {
      bv = best_v[t];
      bi = best_i[t];
    }
  }
  return bi < 0 ? 0 : bi;
}

/*
 * oracle.c — CPU restatement of portBLAS's hot-path algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  Only the test suite, the smoke check and the
 * CPU-baseline leg of the benchmark may load this library, and only as the
 * checker.  The product path (libgbblas.so) never calls it.
 *
 * Every routine states the portBLAS file:line whose semantics it restates
 * (paths relative to the portBLAS source tree).  Inputs arrive as FP64
 * arrays (an exact widening of the FP32 data the GPU sees) so one oracle
 * serves both precisions; accumulation is FP64 with compensation
 * (TwoSum/TwoProd, i.e. double-double) so the oracle is far more accurate
 * than either the reference or the GPU kernels, plus "reference-order" FP32
 * variants that reproduce portBLAS's own arithmetic order.
 *
 * Built with plain gcc (-O2 -fopenmp -ffp-contract=off, no -ffast-math), so
 * the FP32 variants round exactly as written.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <limits.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------ helpers -- */
/* Double-double accumulator: value = hi + lo. */
typedef struct { double hi, lo; } dd_t;

static inline double two_sum(double a, double b, double *e) {
  double s = a + b;
  double bp = s - a;
  double ap = s - bp;
  *e = (a - ap) + (b - bp);
  return s;
}

static inline void dd_add(dd_t *acc, double x) {
  double e;
  double s = two_sum(acc->hi, x, &e);
  double lo = acc->lo + e;
  acc->hi = two_sum(s, lo, &e);
  acc->lo = e;
}

static inline void dd_add_prod(dd_t *acc, double a, double b) {
  double p = a * b;
  double pe = fma(a, b, -p); /* exact product error */
  dd_add(acc, p);
  dd_add(acc, pe);
}

static inline double dd_val(dd_t a) { return a.hi + a.lo; }

/* Element i of a strided view: portBLAS VectorView (src/views/view.hpp:43-48). */
static inline int64_t vidx(int64_t i, int64_t n, int64_t inc) {
  return inc >= 0 ? i * inc : (n - 1 - i) * (-inc);
}

/* --------------------------------------------------------------- GEMM -- */
/*
 * C64 = alpha * op(A) op(B) + beta * C in double-double.
 * Follows Gemm<naive> (src/operations/blas3/gemm_ref.hpp:195-260): one dot
 * product per output, epilogue alpha*acc + beta*C (:240-250); beta == 0 does
 * not read C (src/operations/blas3/gemm_local.hpp:401-409); alpha == 0 scales
 * C by beta and writes zeros when beta == 0
 * (src/interface/gemm_interface.hpp:112-139, blas1_interface.hpp:438-455).
 * Only the entries listed in (rows[s], cols[s]) are computed when nsample >= 0;
 * nsample < 0 computes the whole M x N result into out (column-major, ld M).
 */
void orc_gemm_f64(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const double *A, int64_t lda,
                  const double *B, int64_t ldb, double beta, const double *C, int64_t ldc, int64_t nsample,
                  const int64_t *rows, const int64_t *cols, double *out) {
  int64_t total = nsample >= 0 ? nsample : M * N;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t s = 0; s < total; ++s) {
    int64_t i = nsample >= 0 ? rows[s] : s % M;
    int64_t j = nsample >= 0 ? cols[s] : s / M;
    double c = C ? C[i + j * ldc] : 0.0;
    double r;
    if (alpha == 0.0) {
      r = beta == 0.0 ? 0.0 : beta * c;
    } else {
      dd_t acc = {0.0, 0.0};
      for (int64_t k = 0; k < K; ++k) {
        double a = ta ? A[k + i * lda] : A[i + k * lda];
        double b = tb ? B[j + k * ldb] : B[k + j * ldb];
        dd_add_prod(&acc, a, b);
      }
      dd_t res = {0.0, 0.0};
      dd_add_prod(&res, alpha, acc.hi);
      dd_add_prod(&res, alpha, acc.lo);
      if (beta != 0.0) dd_add_prod(&res, beta, c);
      r = dd_val(res);
    }
    out[s] = r;
  }
}

/*
 * |A|*|B| for the same entries: the componentwise error scale used for the
 * normalised GEMM error |C - C64| / (|alpha| |A||B| + |beta||C|).
 */
void orc_gemm_absscale(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const double *A, int64_t lda,
                       const double *B, int64_t ldb, double beta, const double *C, int64_t ldc, int64_t nsample,
                       const int64_t *rows, const int64_t *cols, double *out) {
  int64_t total = nsample >= 0 ? nsample : M * N;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t s = 0; s < total; ++s) {
    int64_t i = nsample >= 0 ? rows[s] : s % M;
    int64_t j = nsample >= 0 ? cols[s] : s / M;
    double acc = 0.0;
    for (int64_t k = 0; k < K; ++k) {
      double a = ta ? A[k + i * lda] : A[i + k * lda];
      double b = tb ? B[j + k * ldb] : B[k + j * ldb];
      acc += fabs(a) * fabs(b);
    }
    double c = (C && beta != 0.0) ? fabs(beta * C[i + j * ldc]) : 0.0;
    out[s] = fabs(alpha) * acc + c;
  }
}

/*
 * Reference-order FP32 GEMM: sequential FP32 FMA-free accumulation over k as
 * Gemm<naive> does, then either the naive epilogue alpha*acc + beta*C
 * (mode 0, gemm_ref.hpp:248-250) or the Gemm<local> epilogue
 * alpha*(acc + (beta/alpha)*C) (mode 1, gemm_local.hpp:182, 393, 534).
 */
void orc_sgemm_reforder(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha, const float *A, int64_t lda,
                        const float *B, int64_t ldb, float beta, float *C, int64_t ldc, int mode) {
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < N; ++j) {
    for (int64_t i = 0; i < M; ++i) {
      float *cp = C + i + j * ldc;
      if (alpha == 0.0f) {
        *cp = beta == 0.0f ? 0.0f : beta * *cp;
        continue;
      }
      float acc = 0.0f;
      for (int64_t k = 0; k < K; ++k) {
        float a = ta ? A[k + i * lda] : A[i + k * lda];
        float b = tb ? B[j + k * ldb] : B[k + j * ldb];
        float p = a * b;
        acc = acc + p;
      }
      if (mode == 1) {
        float bo = beta / alpha;
        float t = beta == 0.0f ? acc : acc + bo * *cp;
        *cp = alpha * t;
      } else {
        float t = alpha * acc;
        *cp = beta == 0.0f ? t : t + beta * *cp;
      }
    }
  }
}

/* --------------------------------------------------------------- GEMV -- */
/*
 * y64 = alpha * op(A) x + beta * y (double-double).  Follows the naive Gemv
 * form (src/operations/blas2/gemv.hpp:126-172) with the epilogue of
 * src/interface/blas2_interface.hpp:185-211 (beta == 0 does not read y);
 * trans 'n'/'N' is A, anything else A^T (blas2_interface.hpp:1163-1192).
 * out holds the logical y (element i of the view at out[i]).
 */
void orc_gemv_f64(char trans, int64_t M, int64_t N, double alpha, const double *A, int64_t lda, const double *x,
                  int64_t incx, double beta, const double *y, int64_t incy, double *out) {
  int tr = !(trans == 'n' || trans == 'N');
  int64_t xlen = tr ? M : N, ylen = tr ? N : M;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < ylen; ++i) {
    dd_t acc = {0.0, 0.0};
    for (int64_t k = 0; k < xlen; ++k) {
      double a = tr ? A[k + i * lda] : A[i + k * lda];
      dd_add_prod(&acc, a, x[vidx(k, xlen, incx)]);
    }
    dd_t res = {0.0, 0.0};
    dd_add_prod(&res, alpha, acc.hi);
    dd_add_prod(&res, alpha, acc.lo);
    if (beta != 0.0) dd_add_prod(&res, beta, y[vidx(i, ylen, incy)]);
    out[i] = dd_val(res);
  }
}

/* ------------------------------------------------------------- BLAS-1 -- */
/* Parallel double-double sum of f(i) over [0, n): thread partials combined in
 * thread order, so the result is deterministic for a given thread count. */
#define ORC_MAX_THREADS 1024

/* asum: sum |x_i| (AbsoluteAddOperator, src/operations/blas_operators.hpp:257-274;
 * interface src/interface/blas1_interface.hpp:187-246). */
double orc_asum(int64_t n, const double *x, int64_t incx) {
  dd_t parts[ORC_MAX_THREADS];
  int nt = 1;
#pragma omp parallel
  {
#ifdef _OPENMP
    int t = omp_get_thread_num();
#pragma omp single
    nt = omp_get_num_threads();
#else
    int t = 0;
#endif
    dd_t acc = {0.0, 0.0};
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i) dd_add(&acc, fabs(x[vidx(i, n, incx)]));
    if (t < ORC_MAX_THREADS) parts[t] = acc;
  }
  dd_t tot = {0.0, 0.0};
  for (int t = 0; t < nt && t < ORC_MAX_THREADS; ++t) { dd_add(&tot, parts[t].hi); dd_add(&tot, parts[t].lo); }
  return dd_val(tot);
}

/* dot: sum x_i y_i (BinaryOp<Product> + AddOperator,
 * src/interface/blas1_interface.hpp:611-642). */
double orc_dot(int64_t n, const double *x, int64_t incx, const double *y, int64_t incy) {
  dd_t parts[ORC_MAX_THREADS];
  int nt = 1;
#pragma omp parallel
  {
#ifdef _OPENMP
    int t = omp_get_thread_num();
#pragma omp single
    nt = omp_get_num_threads();
#else
    int t = 0;
#endif
    dd_t acc = {0.0, 0.0};
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i) dd_add_prod(&acc, x[vidx(i, n, incx)], y[vidx(i, n, incy)]);
    if (t < ORC_MAX_THREADS) parts[t] = acc;
  }
  dd_t tot = {0.0, 0.0};
  for (int t = 0; t < nt && t < ORC_MAX_THREADS; ++t) { dd_add(&tot, parts[t].hi); dd_add(&tot, parts[t].lo); }
  return dd_val(tot);
}

/* nrm2: sqrt(sum x_i^2) (UnaryOp<Square> + Add then sqrt,
 * src/interface/blas1_interface.hpp:555-579), evaluated with a power-of-two
 * prescale by the largest |x_i| so neither the squares nor the sum over- or
 * underflow; the result is the exactly rounded-to-double norm up to the
 * double-double accumulation error. */
double orc_nrm2(int64_t n, const double *x, int64_t incx) {
  double amax = 0.0;
  int has_nan = 0;
  for (int64_t i = 0; i < n; ++i) {
    double a = fabs(x[vidx(i, n, incx)]);
    if (a != a) has_nan = 1;
    else if (a > amax) amax = a;
  }
  if (has_nan) return NAN;
  if (amax == 0.0) return 0.0;
  if (isinf(amax)) return INFINITY;
  int e;
  frexp(amax, &e);
  double scale = ldexp(1.0, -e); /* exact power of two */
  dd_t parts[ORC_MAX_THREADS];
  int nt = 1;
#pragma omp parallel
  {
#ifdef _OPENMP
    int t = omp_get_thread_num();
#pragma omp single
    nt = omp_get_num_threads();
#else
    int t = 0;
#endif
    dd_t acc = {0.0, 0.0};
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      double v = x[vidx(i, n, incx)] * scale;
      dd_add_prod(&acc, v, v);
    }
    if (t < ORC_MAX_THREADS) parts[t] = acc;
  }
  dd_t tot = {0.0, 0.0};
  for (int t = 0; t < nt && t < ORC_MAX_THREADS; ++t) { dd_add(&tot, parts[t].hi); dd_add(&tot, parts[t].lo); }
  return sqrt(dd_val(tot)) / scale;
}

/*
 * iamax / iamin exactly as IMaxOperator / IMinOperator
 * (src/operations/blas_operators.hpp:276-316) folding from the initial tuple
 * (index INT_MAX, value 0 for max and T max for min:
 * include/operations/blas_constants.h:139-187): the larger (smaller) |x|
 * wins, equal |x| keeps the lower index, NaN never wins.  incx < 0 or n < 0
 * yields 0 (src/interface/blas1_interface.hpp:375-378).  `tmax` is the largest
 * finite value of the element type (FLT_MAX for FP32 data).
 */
int64_t orc_iamax(int64_t n, const double *x, int64_t incx, int is_max, double tmax) {
  if (incx < 0 || n < 0) return 0;
  double bv = is_max ? 0.0 : tmax;
  int64_t bi = INT_MAX;
  for (int64_t i = 0; i < n; ++i) {
    double a = fabs(x[i * incx]);
    int better = is_max ? (a > bv || (a == bv && i < bi)) : (a < bv || (a == bv && i < bi));
    if (better) { bv = a; bi = i; }
  }
  return bi;
}

/* ---------------------------------------------------------- reduction -- */
/*
 * blas::extension::_reduction (src/operations/extension/reduction.hpp:117-230,
 * operators src/operations/blas_operators.hpp:149-274, Mean's two steps
 * src/interface/extension_interface.hpp:46-53).  op: 0 Add, 1 Product, 2 Max,
 * 3 Min, 4 AbsoluteAdd, 5 Mean; dim: 0 inner (per column), 1 outer (per row).
 * Element (i, j) at in[i + j*ld].  Sums are double-double; Product, Max and Min
 * fold in double in index order.  `tmax` is the element type's largest value
 * (Max starts from -tmax = lowest(), Min from tmax).
 */
void orc_reduction(int op, int dim, const double *in, int64_t ld, int64_t rows, int64_t cols, double tmax,
                   double *out) {
  int64_t nout = dim == 0 ? cols : rows;
  int64_t nred = dim == 0 ? rows : cols;
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < nout; ++o) {
    dd_t acc = {0.0, 0.0};
    double v = op == 1 ? 1.0 : (op == 2 ? -tmax : (op == 3 ? tmax : 0.0));
    for (int64_t r = 0; r < nred; ++r) {
      double a = dim == 0 ? in[r + o * ld] : in[o + r * ld];
      switch (op) {
        case 1: v = v * a; break;
        case 2: v = (v > a) ? v : a; break;
        case 3: v = (v < a) ? v : a; break;
        case 4: dd_add(&acc, fabs(a)); break;
        default: dd_add(&acc, a); break;
      }
    }
    if (op == 0 || op == 4) v = dd_val(acc);
    if (op == 5) v = dd_val(acc) / (double)nred;
    out[o] = v;
  }
}

/* Thread count the oracle runs with (for reporting). */
int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

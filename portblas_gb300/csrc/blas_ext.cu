// blas_ext.cu — the element-wise BLAS-1 neighbours of the hot path, the
// matrix copy/transpose extensions and SYMM.
//
//   _scal    x <- alpha*x (alpha == 0 writes zeros: src/interface/blas1_interface.hpp:438-455)
//   _axpy    y <- alpha*x + y
//   _copy    y <- x
//   _sdsdot  rs <- sb + dot(x, y); n == 0 gives sb (blas1_interface.hpp:150-177)
//   extension::_omatcopy   B <- alpha*op(A) (include/interface/extension_interface.h:175-198)
//   extension::_transpose  B <- A^T, out of place or in place through temp memory
//                          (extension_interface.h:405-452)
//   _symm    C <- alpha*A*B + beta*C (side l) or alpha*B*A + beta*C (side r) with
//            A symmetric, one triangle referenced (include/interface/blas3_interface.h:135-145):
//            the referenced triangle is mirrored into a full matrix (a
//            stream-ordered block of its own), then the FP32/FP64 GEMM path
//            (and its selector) runs.
// Vectors follow the strided-view rule of the rest of the library
// (inc < 0 walks from the far end).  All kernels are HBM-bound and read and
// write each element once (transposes through 32x32 shared-memory tiles so
// both sides are coalesced).
#include <cctype>

#include "gemm_internal.cuh"

namespace gb {

// ----------------------------------------------------------- vector maps --
enum : int { kMapScal = 0, kMapAxpy = 1, kMapCopy = 2 };

template <typename T, int OP>
__global__ void vec_map_kernel(int64_t n, T alpha, const T* __restrict__ xb, int64_t incx, T* __restrict__ yb,
                               int64_t incy) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    if (OP == kMapScal) {
      T* p = yb + i * incy;
      *p = alpha == T(0) ? T(0) : alpha * *p;
    } else if (OP == kMapAxpy) {
      T* p = yb + i * incy;
      *p = fma(alpha, xb[i * incx], *p);
    } else {
      yb[i * incy] = xb[i * incx];
    }
  }
}

// contiguous, 16-byte aligned: 128-bit accesses
template <typename T, int OP>
__global__ void vec_map_kernel_v4(int64_t n4, T alpha, const T* __restrict__ x, T* __restrict__ y) {
  using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  constexpr int W = 16 / sizeof(T);
  const V* xv = reinterpret_cast<const V*>(x);
  V* yv = reinterpret_cast<V*>(y);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n4; i += int64_t(gridDim.x) * blockDim.x) {
    V out;
    T* o = reinterpret_cast<T*>(&out);
    if (OP == kMapCopy) {
      out = xv[i];
    } else if (OP == kMapScal) {
      V a = yv[i];
      const T* ap = reinterpret_cast<const T*>(&a);
#pragma unroll
      for (int e = 0; e < W; ++e) o[e] = alpha == T(0) ? T(0) : alpha * ap[e];
    } else {
      V a = xv[i], b = yv[i];
      const T* ap = reinterpret_cast<const T*>(&a);
      const T* bp = reinterpret_cast<const T*>(&b);
#pragma unroll
      for (int e = 0; e < W; ++e) o[e] = fma(alpha, ap[e], bp[e]);
    }
    yv[i] = out;
  }
}

template <typename T, int OP>
gbblas_status_t vec_map(gbblas_handle_t h, int64_t n, T alpha, const T* x, int64_t incx, T* y, int64_t incy) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "null handle");
  if (n <= 0) return GBBLAS_STATUS_SUCCESS;
  if (!y || (OP != kMapScal && !x)) return fail(GBBLAS_STATUS_INVALID_ARG, "null vector");
  const int64_t cap = int64_t(h->sm_count) * 8;
  const bool vec = incy == 1 && aligned16(y) && (OP == kMapScal || (incx == 1 && aligned16(x)));
  if (vec) {
    constexpr int W = 16 / sizeof(T);
    const int64_t n4 = n / W;
    if (n4 > 0) {
      const int64_t blocks = cdiv(n4, 256) < cap ? cdiv(n4, 256) : cap;
      vec_map_kernel_v4<T, OP><<<unsigned(blocks), 256, 0, h->stream>>>(n4, alpha, x, y);
      GB_TRY(after_launch("vec_map_v4"));
    }
    const int64_t rem = n - n4 * W;
    if (rem == 0) return GBBLAS_STATUS_SUCCESS;
    vec_map_kernel<T, OP><<<1, 256, 0, h->stream>>>(rem, alpha, x ? x + n4 * W : nullptr, 1, y + n4 * W, 1);
    return after_launch("vec_map");
  }
  const T* xb = OP == kMapScal ? nullptr : vec_base(x, n, incx);
  T* yb = vec_base(y, n, incy);
  const int64_t blocks = cdiv(n, 256) < cap ? cdiv(n, 256) : cap;
  vec_map_kernel<T, OP><<<unsigned(blocks), 256, 0, h->stream>>>(n, alpha, xb, incx, yb, incy);
  return after_launch("vec_map");
}

__global__ void add_scalar_kernel(float* r, float s) { *r = *r + s; }
__global__ void set_scalar_kernel(float* r, float s) { *r = s; }

// -------------------------------------------------------------- matcopy --
// out(j, i) = alpha * in(i, j) (trans) or out(i, j) = alpha * in(i, j)
template <typename T, bool TRANS>
__global__ void __launch_bounds__(256) matcopy_kernel(int64_t m, int64_t n, T alpha, const T* __restrict__ in,
                                                      int64_t ld_in, T* __restrict__ out, int64_t ld_out) {
  __shared__ T tile[32][33];
  const int64_t i0 = int64_t(blockIdx.x) * 32, j0 = int64_t(blockIdx.y) * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t i = i0 + tx, j = j0 + ty + 8 * q;
    if (i < m && j < n) {
      const T v = alpha * in[i + j * ld_in];
      if (TRANS) tile[ty + 8 * q][tx] = v;
      else out[i + j * ld_out] = v;
    }
  }
  if (!TRANS) return;
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    // out is n x m: out(j, i) at out[j + i*ld_out]; consecutive tx -> consecutive j
    const int64_t j = j0 + tx, i = i0 + ty + 8 * q;
    if (i < m && j < n) out[j + i * ld_out] = tile[tx][ty + 8 * q];
  }
}

template <typename T>
gbblas_status_t matcopy(gbblas_handle_t h, bool trans, int64_t m, int64_t n, T alpha, const T* in, int64_t ld_in,
                        T* out, int64_t ld_out) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "null handle");
  if (m < 0 || n < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "omatcopy: negative dimension");
  if (m == 0 || n == 0) return GBBLAS_STATUS_SUCCESS;
  if (ld_in < m) return fail(GBBLAS_STATUS_INVALID_ARG, "omatcopy: ld_in < m");
  if (ld_out < (trans ? n : m)) return fail(GBBLAS_STATUS_INVALID_ARG, "omatcopy: ld_out too small");
  if (!in || !out) return fail(GBBLAS_STATUS_INVALID_ARG, "omatcopy: null matrix");
  dim3 grid(unsigned(cdiv(m, 32)), unsigned(cdiv(n, 32)));
  if (grid.y > 65535) return fail(GBBLAS_STATUS_UNSUPPORTED, "omatcopy: too many columns");
  if (trans) matcopy_kernel<T, true><<<grid, dim3(32, 8), 0, h->stream>>>(m, n, alpha, in, ld_in, out, ld_out);
  else matcopy_kernel<T, false><<<grid, dim3(32, 8), 0, h->stream>>>(m, n, alpha, in, ld_in, out, ld_out);
  return after_launch("matcopy");
}

// in place through one temp copy: A (m x n, ld_in) -> its transpose (ld_out)
template <typename T>
gbblas_status_t transpose_inplace(gbblas_handle_t h, int64_t m, int64_t n, T* a, int64_t ld_in, int64_t ld_out) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "transpose: null handle");
  if (m < 0 || n < 0 || ld_in < m || ld_out < n) return fail(GBBLAS_STATUS_INVALID_ARG, "transpose: bad shape");
  if (m == 0 || n == 0) return GBBLAS_STATUS_SUCCESS;
  if (!a) return fail(GBBLAS_STATUS_INVALID_ARG, "transpose: null matrix");
  void* tmp;
  GB_TRY(temp_acquire(h, sizeof(T) * size_t(m) * size_t(n), &tmp));
  T* t = static_cast<T*>(tmp);
  GB_TRY(matcopy<T>(h, false, m, n, T(1), a, ld_in, t, m));
  return matcopy<T>(h, true, m, n, T(1), t, m, a, ld_out);
}

// ----------------------------------------------------------------- symm --
// full(i, j) of an order-n symmetric matrix from the referenced triangle
template <typename T>
__global__ void symmetrize_kernel(int64_t n, const T* __restrict__ a, int64_t lda, bool upper, T* __restrict__ full) {
  __shared__ T tile[32][33];
  const int64_t i0 = int64_t(blockIdx.x) * 32, j0 = int64_t(blockIdx.y) * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  // load the mirrored block a(j0.., i0..) transposed, for the elements whose
  // referenced copy is the mirror
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t r = j0 + tx, c = i0 + ty + 8 * q;
    if (r < n && c < n) tile[ty + 8 * q][tx] = a[r + c * lda];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t i = i0 + tx, j = j0 + ty + 8 * q;
    if (i < n && j < n) {
      const bool direct = upper ? (i <= j) : (i >= j);
      full[i + j * n] = direct ? a[i + j * lda] : tile[tx][ty + 8 * q];
    }
  }
}

template <typename T>
gbblas_status_t symm(gbblas_handle_t h, char side, char uplo, int64_t m, int64_t n, T alpha, const T* a,
                     int64_t lda, const T* b, int64_t ldb, T beta, T* c, int64_t ldc) {
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "null handle");
  const char s = char(std::tolower(static_cast<unsigned char>(side)));
  const char u = char(std::tolower(static_cast<unsigned char>(uplo)));
  if (s != 'l' && s != 'r') return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _side");
  if (u != 'u' && u != 'l') return fail(GBBLAS_STATUS_INVALID_ARG, "invalid _uplo");
  if (m < 0 || n < 0) return fail(GBBLAS_STATUS_INVALID_ARG, "symm: negative dimension");
  if (m == 0 || n == 0) return GBBLAS_STATUS_SUCCESS;
  const int64_t na = s == 'l' ? m : n;
  if (lda < na) return fail(GBBLAS_STATUS_INVALID_ARG, "symm: lda < order of A");
  if (!a || !b || !c) return fail(GBBLAS_STATUS_INVALID_ARG, "symm: null matrix");
  dim3 grid(unsigned(cdiv(na, 32)), unsigned(cdiv(na, 32)));
  if (grid.y > 65535) return fail(GBBLAS_STATUS_UNSUPPORTED, "symm: matrix too large");
  // the mirrored matrix gets its own stream-ordered block (the GEMM may grow
  // the handle's temp memory for its own workspace)
  T* full = nullptr;
  GB_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&full), sizeof(T) * size_t(na) * size_t(na), h->stream));
  symmetrize_kernel<T><<<grid, dim3(32, 8), 0, h->stream>>>(na, a, lda, u == 'u', full);
  gbblas_status_t st = after_launch("symmetrize");
  GemmArgs<T> g{};
  g.ta = false;
  g.tb = false;
  g.m = m;
  g.n = n;
  g.alpha = alpha;
  g.beta = beta;
  g.c = c;
  g.ldc = ldc;
  g.batch = 1;
  if (s == 'l') {
    g.k = m;
    g.a = full;
    g.lda = m;
    g.b = b;
    g.ldb = ldb;
  } else {
    g.k = n;
    g.a = b;
    g.lda = ldb;
    g.b = full;
    g.ldb = n;
  }
  if (st == GBBLAS_STATUS_SUCCESS) st = dispatch_gemm(h, g);
  cudaError_t e = cudaFreeAsync(full, h->stream);
  if (st == GBBLAS_STATUS_SUCCESS && e != cudaSuccess) st = cuda_fail(e, "symm: free");
  return st;
}

}  // namespace gb

using namespace gb;

extern "C" {

gbblas_status_t gbblas_sscal(gbblas_handle_t h, int64_t n, float alpha, float* x, int64_t incx) {
  clear_error();
  return vec_map<float, kMapScal>(h, n, alpha, nullptr, 0, x, incx);
}
gbblas_status_t gbblas_dscal(gbblas_handle_t h, int64_t n, double alpha, double* x, int64_t incx) {
  clear_error();
  return vec_map<double, kMapScal>(h, n, alpha, nullptr, 0, x, incx);
}
gbblas_status_t gbblas_saxpy(gbblas_handle_t h, int64_t n, float alpha, const float* x, int64_t incx, float* y,
                             int64_t incy) {
  clear_error();
  return vec_map<float, kMapAxpy>(h, n, alpha, x, incx, y, incy);
}
gbblas_status_t gbblas_daxpy(gbblas_handle_t h, int64_t n, double alpha, const double* x, int64_t incx, double* y,
                             int64_t incy) {
  clear_error();
  return vec_map<double, kMapAxpy>(h, n, alpha, x, incx, y, incy);
}
gbblas_status_t gbblas_scopy(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, float* y, int64_t incy) {
  clear_error();
  return vec_map<float, kMapCopy>(h, n, 0.f, x, incx, y, incy);
}
gbblas_status_t gbblas_dcopy(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, double* y,
                             int64_t incy) {
  clear_error();
  return vec_map<double, kMapCopy>(h, n, 0.0, x, incx, y, incy);
}

gbblas_status_t gbblas_sdsdot(gbblas_handle_t h, int64_t n, float sb, const float* x, int64_t incx, const float* y,
                              int64_t incy, float* result) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "sdsdot: null handle");
  if (!result) return fail(GBBLAS_STATUS_INVALID_ARG, "sdsdot: null result");
  if (n <= 0) {
    set_scalar_kernel<<<1, 1, 0, h->stream>>>(result, sb);
    return after_launch("set_scalar");
  }
  GB_TRY(gbblas_sdot(h, n, x, incx, y, incy, result));
  add_scalar_kernel<<<1, 1, 0, h->stream>>>(result, sb);
  return after_launch("add_scalar");
}

gbblas_status_t gbblas_somatcopy(gbblas_handle_t h, char trans, int64_t m, int64_t n, float alpha, const float* in,
                                 int64_t ld_in, float* out, int64_t ld_out) {
  clear_error();
  return matcopy<float>(h, (trans | 0x20) != 'n', m, n, alpha, in, ld_in, out, ld_out);
}
gbblas_status_t gbblas_domatcopy(gbblas_handle_t h, char trans, int64_t m, int64_t n, double alpha,
                                 const double* in, int64_t ld_in, double* out, int64_t ld_out) {
  clear_error();
  return matcopy<double>(h, (trans | 0x20) != 'n', m, n, alpha, in, ld_in, out, ld_out);
}

gbblas_status_t gbblas_stranspose(gbblas_handle_t h, int64_t m, int64_t n, const float* a, int64_t ld_a, float* b,
                                  int64_t ld_b) {
  clear_error();
  return matcopy<float>(h, true, m, n, 1.f, a, ld_a, b, ld_b);
}
gbblas_status_t gbblas_dtranspose(gbblas_handle_t h, int64_t m, int64_t n, const double* a, int64_t ld_a, double* b,
                                  int64_t ld_b) {
  clear_error();
  return matcopy<double>(h, true, m, n, 1.0, a, ld_a, b, ld_b);
}

gbblas_status_t gbblas_stranspose_inplace(gbblas_handle_t h, int64_t m, int64_t n, float* a, int64_t ld_in,
                                          int64_t ld_out) {
  clear_error();
  return transpose_inplace<float>(h, m, n, a, ld_in, ld_out);
}
gbblas_status_t gbblas_dtranspose_inplace(gbblas_handle_t h, int64_t m, int64_t n, double* a, int64_t ld_in,
                                          int64_t ld_out) {
  clear_error();
  return transpose_inplace<double>(h, m, n, a, ld_in, ld_out);
}

gbblas_status_t gbblas_ssymm(gbblas_handle_t h, char side, char uplo, int64_t m, int64_t n, float alpha,
                             const float* a, int64_t lda, const float* b, int64_t ldb, float beta, float* c,
                             int64_t ldc) {
  clear_error();
  return symm<float>(h, side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc);
}
gbblas_status_t gbblas_dsymm(gbblas_handle_t h, char side, char uplo, int64_t m, int64_t n, double alpha,
                             const double* a, int64_t lda, const double* b, int64_t ldb, double beta, double* c,
                             int64_t ldc) {
  clear_error();
  return symm<double>(h, side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc);
}

}  // extern "C"

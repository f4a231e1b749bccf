/*
 * gbblas.h — C ABI of the GB300-native (sm_103a) BLAS hot path.
 *
 * Every entry point here replaces one portBLAS function on its data-parallel
 * hot path; the portBLAS file:line each one stands in for is given beside it
 * (paths relative to the portBLAS source tree).  The ABI is plain C: opaque
 * handle, plain device pointers, 64-bit sizes and increments, status codes.
 * No CUDA or torch type appears in a signature: a cudaStream_t is passed as
 * `void*`.
 *
 * Conventions shared by every entry point
 *   - All matrices are column-major; element (i, j) of A is A[i + j*lda].
 *   - Vectors follow the portBLAS VectorView rule (src/views/view.hpp:43-48):
 *     with inc > 0 element i is x[i*inc]; with inc < 0 element i is
 *     x[(n-1-i)*|inc|].
 *   - Device pointers only.  Work is enqueued on the handle's stream and the
 *     call returns without waiting (the *_sync variants block and return the
 *     scalar in host memory).
 *   - Results of the BLAS-1 reductions OVERWRITE *result (portBLAS's async
 *     overloads add into it with an atomic; its tests zero it first, so the
 *     results agree).
 *   - Launch errors are reported, never swallowed (portBLAS prints and drops
 *     them: src/sb_handle/kernel_constructor.hpp:213-216).
 */
#ifndef GBBLAS_H
#define GBBLAS_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GBBLAS_STATUS_SUCCESS = 0,
  GBBLAS_STATUS_INVALID_ARG = 1,   /* portBLAS: std::invalid_argument */
  GBBLAS_STATUS_UNSUPPORTED = 2,   /* portBLAS: blas::unsupported_exception */
  GBBLAS_STATUS_CUDA_ERROR = 3,    /* a CUDA runtime / launch error */
  GBBLAS_STATUS_TIMEOUT = 4,       /* a bounded device-side wait gave up */
  GBBLAS_STATUS_ALLOC_FAILED = 5,  /* temp-memory pool could not allocate */
  GBBLAS_STATUS_NOT_INITIALIZED = 6
} gbblas_status_t;

/* blas::extension operators (src/operations/blas_operators.hpp:149-274). */
typedef enum {
  GBBLAS_OP_ADD = 0,
  GBBLAS_OP_PRODUCT = 1,
  GBBLAS_OP_MAX = 2,
  GBBLAS_OP_MIN = 3,
  GBBLAS_OP_ABS_ADD = 4,
  GBBLAS_OP_MEAN = 5
} gbblas_reduction_op_t;

/* blas::reduction_dim_t (include/operations/extension/reduction.h:40):
 * inner reduces each column (output 1 x cols), outer each row (rows x 1). */
typedef enum { GBBLAS_DIM_INNER = 0, GBBLAS_DIM_OUTER = 1 } gbblas_reduction_dim_t;

/* blas::gemm_batch_type_t (include/operations/blas3_trees.h:59). */
typedef enum { GBBLAS_BATCH_STRIDED = 0, GBBLAS_BATCH_INTERLEAVED = 1 } gbblas_batch_type_t;

/* How an FP32 GEMM is computed.  AUTO lets the tile selector choose among the
 * FP32-accurate methods (SIMT or the 3-way BF16 split). */
typedef enum {
  GBBLAS_SGEMM_AUTO = 0,
  GBBLAS_SGEMM_FP32_SIMT = 1,     /* plain FP32 FMA on the CUDA cores */
  GBBLAS_SGEMM_SPLIT_BF16X3 = 2,  /* hi/lo BF16 split, 3 tensor-core products */
  GBBLAS_SGEMM_SPLIT_BF16X6 = 3   /* hi/mid/lo BF16 split, 6 products */
} gbblas_sgemm_mode_t;

/* Element types of the grouped GEMM. */
typedef enum { GBBLAS_DTYPE_F32 = 0, GBBLAS_DTYPE_BF16 = 1, GBBLAS_DTYPE_F64 = 2 } gbblas_dtype_t;

typedef struct gbblas_handle_s* gbblas_handle_t;

/* ---------------------------------------------------------------- handle -- */
/* Replaces blas::SB_Handle(sycl::queue) (include/sb_handle/portblas_handle.h:46-60).
 * `stream` is a cudaStream_t (NULL = legacy default stream).  The handle binds
 * the device that is current at creation. */
gbblas_status_t gbblas_handle_create(void* stream, gbblas_handle_t* handle);
gbblas_status_t gbblas_handle_destroy(gbblas_handle_t handle);
/* Synchronises the old stream before switching, so temp memory in flight on
 * it is never reused on the new one. */
gbblas_status_t gbblas_set_stream(gbblas_handle_t handle, void* stream);
gbblas_status_t gbblas_get_stream(gbblas_handle_t handle, void** stream);
/* Replaces SB_Handle::wait() (include/sb_handle/portblas_handle.h:120-135). */
gbblas_status_t gbblas_wait(gbblas_handle_t handle);
/* Bytes currently held by the handle's stream-ordered temp memory
 * (portBLAS Temp_Mem_Pool statistics, include/sb_handle/temp_memory_pool.h:55-66). */
gbblas_status_t gbblas_temp_bytes(gbblas_handle_t handle, size_t* bytes);
/* Reads and clears the device-side error word (bounded waits that gave up). */
gbblas_status_t gbblas_check_device_error(gbblas_handle_t handle);
/* No portBLAS counterpart: self-test of the device error path.  Launches one
 * CTA that waits on an mbarrier nothing ever arrives at, with the given wall
 * clock limit (capped at 1 s); the wait gives up, records its code in the
 * handle's error word and the kernel returns, leaving the context usable.
 * gbblas_check_device_error then reports GBBLAS_STATUS_TIMEOUT. */
gbblas_status_t gbblas_selftest_wait_timeout(gbblas_handle_t handle, uint64_t limit_ns);
const char* gbblas_status_string(gbblas_status_t status);
/* Message of the last failing call on this thread ("" if none). */
const char* gbblas_last_error(void);
/* Number of kernel launches this library has issued (process-wide). */
uint64_t gbblas_launch_count(void);

gbblas_status_t gbblas_set_sgemm_mode(gbblas_handle_t handle, int mode);
gbblas_status_t gbblas_get_sgemm_mode(gbblas_handle_t handle, int* mode);

/* ---------------------------------------------------------------- BLAS-1 -- */
/* blas::_asum  (include/interface/blas1_interface.h:631-637;
 *               src/interface/blas1_interface.hpp:187-246) */
gbblas_status_t gbblas_sasum(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, float* result);
gbblas_status_t gbblas_dasum(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, double* result);
/* blas::_nrm2  (include/interface/blas1_interface.h:712-718;
 *               src/interface/blas1_interface.hpp:517-581).  Scaled against
 *               overflow/underflow; final scale-and-sqrt in FP64. */
gbblas_status_t gbblas_snrm2(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, float* result);
gbblas_status_t gbblas_dnrm2(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, double* result);
/* blas::_dot   (include/interface/blas1_interface.h:582-588;
 *               src/interface/blas1_interface.hpp:611-642).  n == 0 leaves
 *               *result untouched, as portBLAS does. */
gbblas_status_t gbblas_sdot(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, const float* y,
                            int64_t incy, float* result);
gbblas_status_t gbblas_ddot(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, const double* y,
                            int64_t incy, double* result);
/* blas::_iamax / _iamin (include/interface/blas1_interface.h:646-666;
 *   src/interface/blas1_interface.hpp:278-405; tie rule
 *   src/operations/blas_operators.hpp:276-316).  0-based index of the first
 *   element with the largest (smallest) |x_i|; incx < 0 or n < 0 writes 0;
 *   NaN elements are never selected; when no element qualifies (n == 0) the
 *   index is INT32_MAX, the index of portBLAS's initial tuple. */
gbblas_status_t gbblas_isamax(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, int32_t* result);
gbblas_status_t gbblas_isamin(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, int32_t* result);
gbblas_status_t gbblas_idamax(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, int32_t* result);
gbblas_status_t gbblas_idamin(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, int32_t* result);

/* Synchronous overloads returning the scalar in host memory
 * (include/interface/blas1_interface.h:903-1000;
 *  src/interface/blas1_interface.hpp:1049-1178). */
gbblas_status_t gbblas_sasum_sync(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, float* host_result);
gbblas_status_t gbblas_snrm2_sync(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, float* host_result);
gbblas_status_t gbblas_sdot_sync(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, const float* y,
                                 int64_t incy, float* host_result);
gbblas_status_t gbblas_isamax_sync(gbblas_handle_t h, int64_t n, const float* x, int64_t incx,
                                   int32_t* host_result);
gbblas_status_t gbblas_isamin_sync(gbblas_handle_t h, int64_t n, const float* x, int64_t incx,
                                   int32_t* host_result);
gbblas_status_t gbblas_dasum_sync(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, double* host_result);
gbblas_status_t gbblas_dnrm2_sync(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, double* host_result);
gbblas_status_t gbblas_ddot_sync(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, const double* y,
                                 int64_t incy, double* host_result);
gbblas_status_t gbblas_idamax_sync(gbblas_handle_t h, int64_t n, const double* x, int64_t incx,
                                   int32_t* host_result);
gbblas_status_t gbblas_idamin_sync(gbblas_handle_t h, int64_t n, const double* x, int64_t incx,
                                   int32_t* host_result);

/* Element-wise BLAS-1 neighbours of the hot path (the GEMM alpha == 0
 * shortcut uses the same scaling rule):
 *   _scal  include/interface/blas1_interface.h:697-701  x <- alpha*x (alpha == 0 writes zeros)
 *   _axpy  include/interface/blas1_interface.h:536-541  y <- alpha*x + y
 *   _copy  include/interface/blas1_interface.h:556-560  y <- x
 *   _sdsdot include/interface/blas1_interface.h:615-620 result <- sb + dot(x, y) (n == 0: sb) */
gbblas_status_t gbblas_sscal(gbblas_handle_t h, int64_t n, float alpha, float* x, int64_t incx);
gbblas_status_t gbblas_dscal(gbblas_handle_t h, int64_t n, double alpha, double* x, int64_t incx);
gbblas_status_t gbblas_saxpy(gbblas_handle_t h, int64_t n, float alpha, const float* x, int64_t incx, float* y,
                             int64_t incy);
gbblas_status_t gbblas_daxpy(gbblas_handle_t h, int64_t n, double alpha, const double* x, int64_t incx, double* y,
                             int64_t incy);
gbblas_status_t gbblas_scopy(gbblas_handle_t h, int64_t n, const float* x, int64_t incx, float* y, int64_t incy);
gbblas_status_t gbblas_dcopy(gbblas_handle_t h, int64_t n, const double* x, int64_t incx, double* y,
                             int64_t incy);
gbblas_status_t gbblas_sdsdot(gbblas_handle_t h, int64_t n, float sb, const float* x, int64_t incx, const float* y,
                              int64_t incy, float* result);

/* ---------------------------------------------------------------- BLAS-2 -- */
/* blas::_gemv  (include/interface/blas2_interface.h:632-655;
 *   src/interface/blas2_interface.hpp:68-217, 1163-1192).
 *   y <- alpha*op(A)*x + beta*y; trans 'n'/'N' is op(A)=A, anything else A^T.
 *   beta == 0 never reads y. */
gbblas_status_t gbblas_sgemv(gbblas_handle_t h, char trans, int64_t m, int64_t n, float alpha, const float* a,
                             int64_t lda, const float* x, int64_t incx, float beta, float* y, int64_t incy);
gbblas_status_t gbblas_dgemv(gbblas_handle_t h, char trans, int64_t m, int64_t n, double alpha, const double* a,
                             int64_t lda, const double* x, int64_t incx, double beta, double* y, int64_t incy);

/* Allocation-free GEMV.  No counterpart in portBLAS: it is gbblas_sgemv for
 * callers that cannot allocate device memory — hosts whose device memory is
 * owned by their own allocator, plug-in hosts that forbid allocation once
 * running, latency-critical loops that cannot take cudaMalloc's implicit
 * synchronisation.  Same arguments and results as gbblas_sgemv, but it takes
 * the cudaStream_t directly (no handle; the stream must belong to the current
 * device) and its scratch is a fixed 1 MiB block of file-scope device memory
 * (plus 256 KiB of ticket counters) that every GPU loading the library holds
 * until exit.  Argument errors are rejected before anything is enqueued; a
 * problem needing more scratch is rejected with GBBLAS_STATUS_INVALID_ARG
 * before any kernel runs.  Each call enqueues one cudaMemsetAsync clearing
 * 4 bytes of tickets per output element (at most 256 KiB).  The first call on
 * a device looks the block's address up (cudaGetSymbolAddress, a synchronous
 * runtime call).  All calls share the block, so calls that overlap on the
 * GPU race.  A device-side wait that gives up (2 s) is not reported by this
 * call (it has returned SUCCESS; y may be wrong): use gbblas_sgemv with a
 * handle and gbblas_check_device_error where that must be seen. */
gbblas_status_t gbblas_sgemv_noalloc(void* stream, char trans, int64_t m, int64_t n, float alpha, const float* a,
                                     int64_t lda, const float* x, int64_t incx, float beta, float* y,
                                     int64_t incy);

/* ---------------------------------------------------------------- BLAS-3 -- */
/* blas::_gemm  (include/interface/blas3_interface.h:86-95;
 *   src/interface/gemm_interface.hpp:102-198).
 *   C <- alpha*op(A)*op(B) + beta*C; trans in {n,t,c} (any case, c == t for
 *   real types).  alpha == 0 scales C by beta without reading A or B
 *   (beta == 0 writes zeros); beta == 0 never reads C. */
gbblas_status_t gbblas_sgemm(gbblas_handle_t h, char transa, char transb, int64_t m, int64_t n, int64_t k,
                             float alpha, const float* a, int64_t lda, const float* b, int64_t ldb, float beta,
                             float* c, int64_t ldc);
gbblas_status_t gbblas_dgemm(gbblas_handle_t h, char transa, char transb, int64_t m, int64_t n, int64_t k,
                             double alpha, const double* a, int64_t lda, const double* b, int64_t ldb,
                             double beta, double* c, int64_t ldc);
/* blas::_gemm_batched (include/interface/blas3_interface.h:97-109;
 *   src/interface/gemm_interface.hpp:200-226).  Strided batch with the
 *   default strides (ta? m*lda : k*lda), (tb? ldb*k : n*ldb), ldc*n; the
 *   interleaved batch type keeps batch as the fastest axis: element (r, c)
 *   of matrix b is at ptr[(r + c*ld)*batch + b]. */
gbblas_status_t gbblas_sgemm_batched(gbblas_handle_t h, char transa, char transb, int64_t m, int64_t n,
                                     int64_t k, float alpha, const float* a, int64_t lda, const float* b,
                                     int64_t ldb, float beta, float* c, int64_t ldc, int64_t batch_size,
                                     int batch_type);
gbblas_status_t gbblas_dgemm_batched(gbblas_handle_t h, char transa, char transb, int64_t m, int64_t n,
                                     int64_t k, double alpha, const double* a, int64_t lda, const double* b,
                                     int64_t ldb, double beta, double* c, int64_t ldc, int64_t batch_size,
                                     int batch_type);
/* blas::_gemm_strided_batched (include/interface/blas3_interface.h:111-123;
 *   src/interface/gemm_interface.hpp:228-240).  stride_a / stride_b may be 0;
 *   stride_c < ldc*n or any negative stride is INVALID_ARG (:153-166). */
gbblas_status_t gbblas_sgemm_strided_batched(gbblas_handle_t h, char transa, char transb, int64_t m, int64_t n,
                                             int64_t k, float alpha, const float* a, int64_t lda,
                                             int64_t stride_a, const float* b, int64_t ldb, int64_t stride_b,
                                             float beta, float* c, int64_t ldc, int64_t stride_c,
                                             int64_t batch_size);
gbblas_status_t gbblas_dgemm_strided_batched(gbblas_handle_t h, char transa, char transb, int64_t m, int64_t n,
                                             int64_t k, double alpha, const double* a, int64_t lda,
                                             int64_t stride_a, const double* b, int64_t ldb, int64_t stride_b,
                                             double beta, double* c, int64_t ldc, int64_t stride_c,
                                             int64_t batch_size);

/* blas::_symm (include/interface/blas3_interface.h:135-145): C <- alpha*A*B +
 * beta*C (side 'l', A m x m) or alpha*B*A + beta*C (side 'r', A n x n), A
 * symmetric with only the `uplo` ('u'/'l') triangle referenced. */
gbblas_status_t gbblas_ssymm(gbblas_handle_t h, char side, char uplo, int64_t m, int64_t n, float alpha,
                             const float* a, int64_t lda, const float* b, int64_t ldb, float beta, float* c,
                             int64_t ldc);
gbblas_status_t gbblas_dsymm(gbblas_handle_t h, char side, char uplo, int64_t m, int64_t n, double alpha,
                             const double* a, int64_t lda, const double* b, int64_t ldb, double beta, double* c,
                             int64_t ldc);

/* GEMM tile configurations (no portBLAS counterpart: portBLAS fixes its
 * tile at compile time from size thresholds per element type,
 * src/interface/blas3/backend/nvidia_gpu.hpp:116-171).  FP32: configs 0..19
 * are SIMT tiles {128x128, 128x64, 64x128, 64x64} x split-K {1,2,4,8,16},
 * 20..39 the 3-term split-BF16 tcgen05 kernel with N tile {128, 64} x
 * split-K {1,2,4,8,16} x raster (raster_m 2: groups of 16 tile rows down M,
 * then along N; 1: down M); all are FP32-accurate.  FP64:
 * configs 40..59 are SIMT tiles x split-K as 0..19.  AUTO picks one of the
 * element type's configs per call (autotuned winner > learned selector >
 * size heuristic).  config_info takes any config (method 0 FP32 SIMT,
 * 1 split-BF16, 2 FP64 SIMT); sgemm_config_count is 40 (FP32), gemm_config_
 * count 60 (all). */
int gbblas_sgemm_config_count(void);
int gbblas_gemm_config_count(void);
gbblas_status_t gbblas_sgemm_config_info(int config, int* method, int* tile_m, int* tile_n, int* split,
                                         int* raster_m);
gbblas_status_t gbblas_sgemm_strided_batched_config(gbblas_handle_t h, int config, char transa, char transb,
                                                    int64_t m, int64_t n, int64_t k, float alpha, const float* a,
                                                    int64_t lda, int64_t stride_a, const float* b, int64_t ldb,
                                                    int64_t stride_b, float beta, float* c, int64_t ldc,
                                                    int64_t stride_c, int64_t batch_size);
gbblas_status_t gbblas_dgemm_strided_batched_config(gbblas_handle_t h, int config, char transa, char transb,
                                                    int64_t m, int64_t n, int64_t k, double alpha, const double* a,
                                                    int64_t lda, int64_t stride_a, const double* b, int64_t ldb,
                                                    int64_t stride_b, double beta, double* c, int64_t ldc,
                                                    int64_t stride_c, int64_t batch_size);
/* Selector inputs: log2 M, N, K (/14), transa, transb, lda/ldb/ldc mod 16
 * (/16), log2 batch (/10), element type one-hot (FP32, FP64) — 11 floats.
 * dtype is GBBLAS_DTYPE_F32 or GBBLAS_DTYPE_F64; the sgemm_ forms are FP32. */
gbblas_status_t gbblas_gemm_features(int dtype, int64_t m, int64_t n, int64_t k, char transa, char transb,
                                     int64_t lda, int64_t ldb, int64_t ldc, int64_t batch, float* features);
gbblas_status_t gbblas_sgemm_features(int64_t m, int64_t n, int64_t k, char transa, char transb, int64_t lda,
                                      int64_t ldb, int64_t ldc, int64_t batch, float* features);
/* The fixed size-threshold selector alone (portBLAS-style tiers). */
int gbblas_gemm_heuristic_config(int dtype, int64_t m, int64_t n, int64_t k, int64_t batch);
int gbblas_sgemm_heuristic_config(int64_t m, int64_t n, int64_t k, int64_t batch);
/* Loads learned-selector weights (process-wide; default file
 * tuning/gemm_selector.bin beside the package, or $GBBLAS_SGEMM_SELECTOR,
 * "off" disables), and asks the selector chain for a config of the element
 * type. */
gbblas_status_t gbblas_sgemm_load_selector(const char* path);
gbblas_status_t gbblas_gemm_selector_pick(int dtype, int64_t m, int64_t n, int64_t k, char transa, char transb,
                                          int64_t lda, int64_t ldb, int64_t ldc, int64_t batch, int* config);
gbblas_status_t gbblas_sgemm_selector_pick(int64_t m, int64_t n, int64_t k, char transa, char transb, int64_t lda,
                                           int64_t ldb, int64_t ldc, int64_t batch, int* config);
/* No portBLAS counterpart: the tiles the fixed split-BF16 modes (`mode`
 * GBBLAS_SGEMM_SPLIT_BF16X3 or _X6) run an m x n x k GEMM of `batch`
 * matrices on, for a GPU with `sm_count` SMs, computed on the host (no device
 * call).  `tile_m` x `tile_n`: the output tile of one work item (tile_m 256:
 * a CTA pair sharing one tile); `k_slices`: split-K slices (1: no split).
 * Any output pointer may be null. */
gbblas_status_t gbblas_sgemm_split_route(int64_t m, int64_t n, int64_t k, int64_t batch, int mode, int sm_count,
                                         int* tile_m, int* tile_n, int* k_slices);
/* Exhaustive autotune of one shape: times every config of the element type
 * (`reps` launches each) on zero-filled operands, remembers the winner for
 * AUTO. */
gbblas_status_t gbblas_sgemm_autotune(gbblas_handle_t h, char transa, char transb, int64_t m, int64_t n,
                                      int64_t k, int64_t lda, int64_t ldb, int64_t ldc, int64_t batch, int reps,
                                      int* best_config, float* best_ms);
gbblas_status_t gbblas_dgemm_autotune(gbblas_handle_t h, char transa, char transb, int64_t m, int64_t n,
                                      int64_t k, int64_t lda, int64_t ldb, int64_t ldc, int64_t batch, int reps,
                                      int* best_config, float* best_ms);

/* Training and inference kernels of the learned selector (no portBLAS
 * counterpart).  Network in -> hidden x3 (GELU) -> out, FP32, parameters
 * packed [W1 b1 W2 b2 W3 b3 W4 b4] (W row-major out x in) in device memory;
 * x is [n][in], y / target / mask are [n][out].  loss_grad writes the
 * gradients of the masked MSE (sum over mask / valid_count) and the loss
 * (device scalar); adam applies one AdamW step. */
gbblas_status_t gbblas_mlp_param_count(int in_dim, int hidden, int out_dim, int64_t* count);
gbblas_status_t gbblas_mlp_forward(gbblas_handle_t h, int in_dim, int hidden, int out_dim, const float* params,
                                   const float* x, int64_t n, float* y);
gbblas_status_t gbblas_mlp_loss_grad(gbblas_handle_t h, int in_dim, int hidden, int out_dim, const float* params,
                                     const float* x, const float* target, const float* mask, int64_t n,
                                     float valid_count, float* grads, float* loss);
gbblas_status_t gbblas_mlp_adam(gbblas_handle_t h, int64_t count, float* params, const float* grads, float* m,
                                float* v, int step, float lr, float beta1, float beta2, float eps,
                                float weight_decay);

/* Grouped GEMM over `count` independent problems of uneven sizes, one
 * persistent launch with a device-side tile scheduler.  No portBLAS
 * counterpart takes uneven sizes; per problem the semantics are those of
 * blas::_gemm (src/interface/gemm_interface.hpp:102-198).  All arrays are
 * HOST arrays of length `count`; a/b/c hold device pointers.  `dtype` is the
 * element type of A and B (F32 or BF16); C is always FP32 and accumulation is
 * FP32.  The problem table is uploaded into the handle's temp memory. */
gbblas_status_t gbblas_gemm_grouped(gbblas_handle_t h, int dtype, int64_t count, const char* transa,
                                    const char* transb, const int64_t* m, const int64_t* n, const int64_t* k,
                                    const float* alpha, const void* const* a, const int64_t* lda,
                                    const void* const* b, const int64_t* ldb, const float* beta, float* const* c,
                                    const int64_t* ldc);

/* A reusable grouped GEMM: the problem table is uploaded once and every run
 * replays one CUDA graph holding the persistent launch (no host work per
 * run beyond cudaGraphLaunch).  Pointers and sizes are fixed at creation;
 * the data behind them may change between runs.  After a run that
 * gbblas_check_device_error reports as timed out, destroy and re-create the
 * plan (its device counters may not have been reset). */
typedef struct gbblas_grouped_plan_s* gbblas_grouped_plan_t;
gbblas_status_t gbblas_grouped_plan_create(gbblas_handle_t h, int dtype, int64_t count, const char* transa,
                                           const char* transb, const int64_t* m, const int64_t* n,
                                           const int64_t* k, const float* alpha, const void* const* a,
                                           const int64_t* lda, const void* const* b, const int64_t* ldb,
                                           const float* beta, float* const* c, const int64_t* ldc,
                                           gbblas_grouped_plan_t* plan);
gbblas_status_t gbblas_grouped_plan_run(gbblas_handle_t h, gbblas_grouped_plan_t plan);
gbblas_status_t gbblas_grouped_plan_destroy(gbblas_grouped_plan_t plan);
/* No portBLAS counterpart: the plan's schedule.  `tiles`: tiles the
 * persistent kernel hands out (output tiles x K slices); `max_splits`: the
 * largest number of K slices of any problem (1: no split-K).  Either output
 * pointer may be null. */
gbblas_status_t gbblas_grouped_plan_info(gbblas_grouped_plan_t plan, int64_t* tiles, int* max_splits);
/* No portBLAS counterpart: the tile schedule a tcgen05 grouped plan of these
 * problems would use on a GPU with `sm_count` SMs, computed on the host (no
 * device call).  `tiles`: tiles handed out; `splits[i]` (host array of
 * `count`): K slices of problem i, 0 for a problem with m or n == 0. */
gbblas_status_t gbblas_grouped_schedule(int dtype, int64_t count, const char* transa, const char* transb,
                                        const int64_t* m, const int64_t* n, const int64_t* k, const float* alpha,
                                        int sm_count, int64_t* tiles, int* splits);

/* ------------------------------------------------------------ extension -- */
/* blas::extension::_omatcopy (include/interface/extension_interface.h:188-198):
 * out <- alpha * op(in); in is m x n, out is m x n ('n') or n x m ('t'/'c'). */
gbblas_status_t gbblas_somatcopy(gbblas_handle_t h, char trans, int64_t m, int64_t n, float alpha, const float* in,
                                 int64_t ld_in, float* out, int64_t ld_out);
gbblas_status_t gbblas_domatcopy(gbblas_handle_t h, char trans, int64_t m, int64_t n, double alpha,
                                 const double* in, int64_t ld_in, double* out, int64_t ld_out);
/* blas::extension::_transpose (include/interface/extension_interface.h:405-452):
 * out of place B <- A^T (A m x n), and in place (A reinterpreted from ld_in to
 * its n x m transpose with ld_out, through temp memory). */
gbblas_status_t gbblas_stranspose(gbblas_handle_t h, int64_t m, int64_t n, const float* a, int64_t ld_a, float* b,
                                  int64_t ld_b);
gbblas_status_t gbblas_stranspose_inplace(gbblas_handle_t h, int64_t m, int64_t n, float* a, int64_t ld_in,
                                          int64_t ld_out);
gbblas_status_t gbblas_dtranspose(gbblas_handle_t h, int64_t m, int64_t n, const double* a, int64_t ld_a, double* b,
                                  int64_t ld_b);
gbblas_status_t gbblas_dtranspose_inplace(gbblas_handle_t h, int64_t m, int64_t n, double* a, int64_t ld_in,
                                          int64_t ld_out);

/* blas::extension::_reduction<op, T> (include/interface/extension_interface.h:453-462;
 *   src/interface/extension_interface.hpp:344-409, 578-593;
 *   src/operations/extension/reduction.hpp:35-236).
 *   in is rows x cols with leading dimension ld (ld >= rows); out has cols
 *   elements (inner) or rows elements (outer).  Mean divides by the reduced
 *   length. */
gbblas_status_t gbblas_sreduction(gbblas_handle_t h, int op, int dim, const float* in, int64_t ld, float* out,
                                  int64_t rows, int64_t cols);
gbblas_status_t gbblas_dreduction(gbblas_handle_t h, int op, int dim, const double* in, int64_t ld, double* out,
                                  int64_t rows, int64_t cols);

#ifdef __cplusplus
}
#endif

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#endif /* GBBLAS_H */

// common.cuh — shared host/device helpers of the gbblas library.
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <cstddef>
#include <mutex>
#include <string>
#include <utility>

#include "../../include/gbblas.h"

namespace gb {

// ----------------------------------------------------------------- errors --
// Per-thread message of the last failing call (gbblas_last_error).
void set_error(const std::string& msg);
void clear_error();

struct Status {
  gbblas_status_t code = GBBLAS_STATUS_SUCCESS;
};

inline gbblas_status_t fail(gbblas_status_t code, const std::string& msg) {
  set_error(msg);
  return code;
}

inline gbblas_status_t cuda_fail(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return GBBLAS_STATUS_CUDA_ERROR;
}

#define GB_CUDA_TRY(expr)                                   \
  do {                                                      \
    cudaError_t _e = (expr);                                \
    if (_e != cudaSuccess) return ::gb::cuda_fail(_e, #expr); \
  } while (0)

#define GB_TRY(expr)                                         \
  do {                                                       \
    gbblas_status_t _s = (expr);                             \
    if (_s != GBBLAS_STATUS_SUCCESS) return _s;              \
  } while (0)

// Checks the launch that was just issued and counts it.
gbblas_status_t after_launch(const char* kernel);

// ----------------------------------------------------------------- handle --
}  // namespace gb

struct gbblas_handle_s {
  cudaStream_t stream = nullptr;
  int device = 0;
  int sm_count = 0;
  int max_smem_optin = 0;
  // Stream-ordered temp memory: one growable block, released with
  // cudaFreeAsync on the same stream (the portBLAS Temp_Mem_Pool equivalent,
  // include/sb_handle/temp_memory_pool.h:33-114).
  void* temp = nullptr;
  size_t temp_size = 0;
  // Zero-initialised ticket counters used by the last-block-done reductions.
  // Every kernel that takes tickets resets the ones it used before exiting.
  unsigned int* tickets = nullptr;
  size_t n_tickets = 0;
  // Device error word written by bounded waits that gave up.
  int* dev_error = nullptr;
  // Pinned host staging for the *_sync overloads.
  void* pinned = nullptr;
  int sgemm_mode = GBBLAS_SGEMM_AUTO;
  // set for the allocation-free entry point: temp memory is a fixed block and
  // a request beyond it is an error instead of a cudaMallocAsync
  bool no_alloc = false;
  std::mutex mu;  // guards temp memory, as the portBLAS pool mutex does
};

namespace gb {

// Returns a device pointer to at least `bytes` of temp memory, 256-byte aligned.
// Stream-ordered: the block stays valid for everything enqueued afterwards on
// the handle's stream until the next call that grows it.
gbblas_status_t temp_acquire(gbblas_handle_t h, size_t bytes, void** ptr);
// Number of ticket counters available: kMaxTickets.
constexpr size_t kMaxTickets = 1u << 16;

__host__ __device__ inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Element i of a strided vector view (portBLAS VectorView, src/views/view.hpp:43-48).
template <typename T>
__host__ __device__ __forceinline__ const T* vec_base(const T* x, int64_t n, int64_t inc) {
  return inc >= 0 ? x : x + (n - 1) * (-inc);
}
template <typename T>
__host__ __device__ __forceinline__ T* vec_base(T* x, int64_t n, int64_t inc) {
  return inc >= 0 ? x : x + (n - 1) * (-inc);
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Raises `func`'s dynamic shared-memory limit to `bytes` on device `dev`.
// The attribute belongs to each device's context, so a process driving
// several GPUs must set it on every one: `done` is the call site's mask with
// one bit per device (0..63; higher devices set it on every call).  Two
// threads that race on a first call both set it, which is harmless.
inline cudaError_t raise_smem_limit(std::atomic<uint64_t>& done, const void* func, int bytes, int dev) {
  const uint64_t bit = (dev >= 0 && dev < 64) ? (uint64_t(1) << dev) : 0;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

// ------------------------------------------------ programmatic dependent launch --
// A kernel launched with launch_pdl(..., early = true) may place its CTAs and
// run up to pdl_wait() while the previous kernel on the stream drains;
// pdl_wait() returns once every earlier grid on the stream has completed with
// its writes visible, so stream order is kept.  It is used only for grids of
// exactly one full wave (every SM at its resident-CTA limit), whose early
// placement cannot come out uneven.  Both calls are no-ops for a normal
// launch; GBBLAS_PDL=0 in the environment turns early launch off.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

bool pdl_enabled();

// Brings `bytes` bytes from p into L2 (p 16-byte aligned, bytes a multiple
// of 16).  A prefetch is only a hint: it changes no value any thread reads
// (L2 is where every SM's loads and stores meet), so a kernel may warm its
// first inputs before pdl_wait(), while the previous kernel on the stream is
// still draining.
__device__ __forceinline__ void prefetch_l2_bulk(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(reinterpret_cast<uint64_t>(p)), "r"(bytes)
               : "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(bool early, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t s, Args&&... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = (early && pdl_enabled()) ? 1 : 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace gb

// handle.cu — SB_Handle equivalent: stream binding, stream-ordered temp
// memory, error reporting.  Replaces blas::SB_Handle and Temp_Mem_Pool
// (include/sb_handle/portblas_handle.h:46-200,
//  src/sb_handle/portblas_handle.hpp:42-100,
//  include/sb_handle/temp_memory_pool.h:33-114).
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <new>

#include "common.cuh"
#include "tc_ptx.cuh"

namespace gb {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

void set_error(const std::string& msg) { g_last_error = msg; }

bool pdl_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("GBBLAS_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}
void clear_error() { g_last_error.clear(); }

gbblas_status_t after_launch(const char* kernel) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, kernel);
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t temp_acquire(gbblas_handle_t h, size_t bytes, void** ptr) {
  std::lock_guard<std::mutex> lk(h->mu);
  bytes = (bytes + 255) & ~size_t(255);
  if (bytes == 0) bytes = 256;
  if (bytes > h->temp_size) {
    if (h->no_alloc)
      return fail(GBBLAS_STATUS_INVALID_ARG, "problem needs " + std::to_string(bytes) +
                                                 " bytes of scratch, above the allocation-free maximum of " +
                                                 std::to_string(h->temp_size) + " bytes");
    size_t grow = h->temp_size * 2 > bytes ? h->temp_size * 2 : bytes;
    if (h->temp) {
      cudaError_t e = cudaFreeAsync(h->temp, h->stream);
      h->temp = nullptr;
      h->temp_size = 0;
      if (e != cudaSuccess) return cuda_fail(e, "cudaFreeAsync(temp)");
    }
    cudaError_t e = cudaMallocAsync(&h->temp, grow, h->stream);
    if (e != cudaSuccess) {
      h->temp = nullptr;
      set_error(std::string("temp memory: cudaMallocAsync failed: ") + cudaGetErrorString(e));
      return GBBLAS_STATUS_ALLOC_FAILED;
    }
    h->temp_size = grow;
  }
  *ptr = h->temp;
  return GBBLAS_STATUS_SUCCESS;
}

// Waits on an mbarrier that never completes (phase 0, no arrivals) until the
// bounded wait gives up, then records the error code and returns.
constexpr int kErrSelftest = 901;
__global__ void selftest_timeout_kernel(int* err, uint64_t limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && !tc::mbar_wait(&bar, 0, limit_ns)) atomicExch(err, kErrSelftest);
}

}  // namespace gb

using namespace gb;

extern "C" {

const char* gbblas_last_error(void) { return g_last_error.c_str(); }

uint64_t gbblas_launch_count(void) { return g_launches.load(); }

const char* gbblas_status_string(gbblas_status_t s) {
  switch (s) {
    case GBBLAS_STATUS_SUCCESS: return "success";
    case GBBLAS_STATUS_INVALID_ARG: return "invalid argument";
    case GBBLAS_STATUS_UNSUPPORTED: return "unsupported";
    case GBBLAS_STATUS_CUDA_ERROR: return "CUDA error";
    case GBBLAS_STATUS_TIMEOUT: return "device wait timed out";
    case GBBLAS_STATUS_ALLOC_FAILED: return "temp memory allocation failed";
    case GBBLAS_STATUS_NOT_INITIALIZED: return "handle not initialized";
  }
  return "unknown status";
}

gbblas_status_t gbblas_handle_create(void* stream, gbblas_handle_t* out) {
  clear_error();
  if (!out) return fail(GBBLAS_STATUS_INVALID_ARG, "handle_create: null output pointer");
  *out = nullptr;
  gbblas_handle_s* h = new (std::nothrow) gbblas_handle_s();
  if (!h) return fail(GBBLAS_STATUS_ALLOC_FAILED, "handle_create: out of host memory");
  h->stream = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&h->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  if (e == cudaSuccess) e = cudaMalloc(&h->tickets, kMaxTickets * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(h->tickets, 0, kMaxTickets * sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc(&h->dev_error, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(h->dev_error, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMallocHost(&h->pinned, 64);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    gbblas_handle_destroy(h);
    return cuda_fail(e, "handle_create");
  }
  h->n_tickets = kMaxTickets;
  *out = h;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_handle_destroy(gbblas_handle_t h) {
  if (!h) return GBBLAS_STATUS_SUCCESS;
  cudaStreamSynchronize(h->stream);
  if (h->temp) cudaFree(h->temp);
  if (h->tickets) cudaFree(h->tickets);
  if (h->dev_error) cudaFree(h->dev_error);
  if (h->pinned) cudaFreeHost(h->pinned);
  delete h;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_set_stream(gbblas_handle_t h, void* stream) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "set_stream: null handle");
  GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->stream = static_cast<cudaStream_t>(stream);
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_get_stream(gbblas_handle_t h, void** stream) {
  if (!h || !stream) return fail(GBBLAS_STATUS_INVALID_ARG, "get_stream: null argument");
  *stream = h->stream;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_wait(gbblas_handle_t h) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "wait: null handle");
  GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_temp_bytes(gbblas_handle_t h, size_t* bytes) {
  if (!h || !bytes) return fail(GBBLAS_STATUS_INVALID_ARG, "temp_bytes: null argument");
  *bytes = h->temp_size;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_check_device_error(gbblas_handle_t h) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "check_device_error: null handle");
  int flag = 0;
  GB_CUDA_TRY(cudaMemcpyAsync(&flag, h->dev_error, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  GB_CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (flag) {
    GB_CUDA_TRY(cudaMemsetAsync(h->dev_error, 0, sizeof(int), h->stream));
    return fail(GBBLAS_STATUS_TIMEOUT, "a bounded device-side wait gave up (code " + std::to_string(flag) + ")");
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_selftest_wait_timeout(gbblas_handle_t h, uint64_t limit_ns) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "selftest: null handle");
  if (limit_ns > 1000000000ull) limit_ns = 1000000000ull;
  selftest_timeout_kernel<<<1, 32, 0, h->stream>>>(h->dev_error, limit_ns);
  return after_launch("selftest_timeout");
}

gbblas_status_t gbblas_set_sgemm_mode(gbblas_handle_t h, int mode) {
  clear_error();
  if (!h) return fail(GBBLAS_STATUS_NOT_INITIALIZED, "set_sgemm_mode: null handle");
  if (mode < GBBLAS_SGEMM_AUTO || mode > GBBLAS_SGEMM_SPLIT_BF16X6)
    return fail(GBBLAS_STATUS_INVALID_ARG, "set_sgemm_mode: unknown mode");
  h->sgemm_mode = mode;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status_t gbblas_get_sgemm_mode(gbblas_handle_t h, int* mode) {
  if (!h || !mode) return fail(GBBLAS_STATUS_INVALID_ARG, "get_sgemm_mode: null argument");
  *mode = h->sgemm_mode;
  return GBBLAS_STATUS_SUCCESS;
}

}  // extern "C"

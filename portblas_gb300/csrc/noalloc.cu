// noalloc.cu — a GEMV entry point that allocates no device memory.
//
// Some callers cannot allocate device memory: hosts whose device memory is
// fully carved up by their own allocator (a framework's caching allocator, a
// pool sized at start-up), plug-in hosts that forbid allocation once running,
// and latency-critical loops that cannot take the implicit synchronisation of
// cudaMalloc/cudaFree.  gbblas_sgemv_noalloc serves them.  It runs the same
// GEMV kernels as gbblas_sgemv, but the scratch those kernels need (the split
// partial sums and the last-CTA tickets) lives in file-scope __device__
// arrays of fixed size, and the handle is built on the stack around the
// caller's stream.
//
// Limits and rules (also stated in include/gbblas.h):
//   * scratch: kNoAllocScratchBytes (1 MiB) of partial sums; a problem whose
//     split plan needs more is rejected with GBBLAS_STATUS_INVALID_ARG before
//     any kernel runs (argument errors are rejected before anything is
//     enqueued; the ticket clear below may already be enqueued for a problem
//     rejected for its scratch size, which changes nothing but the tickets);
//   * every GPU that loads the library holds the arrays (1 MiB + 256 KiB)
//     until the process exits;
//   * the first call on each device looks up the arrays' device addresses
//     (cudaGetSymbolAddress with that device current, a synchronous runtime
//     call);
//   * the stream must belong to the current device (INVALID_ARG otherwise);
//   * all calls share the arrays: calls that overlap on the GPU (different
//     streams, no ordering between them) race and give wrong results;
//   * each call clears the tickets it can use (one cudaMemsetAsync of
//     4 bytes per output element, at most 256 KiB) so that a call that failed
//     on the device cannot leave the next one a non-zero count; the partial
//     sums need no clearing;
//   * a bounded device-side wait that gives up (a TMA copy that does not land
//     within 2 s) is recorded in a per-device word that this entry point does
//     not report: the call has already returned SUCCESS and y may be wrong.
//     Callers that need such timeouts reported use gbblas_sgemv with a handle
//     and gbblas_check_device_error.
#include <mutex>

#include "common.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(1) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
static __device__ __align__(256) unsigned int g_noalloc_tickets[gb::kMaxTickets];
static __device__ __align__(256) int g_noalloc_error;

struct DeviceArrays {
  bool ready = false;
  void* scratch = nullptr;
  unsigned int* tickets = nullptr;
  int* error = nullptr;
  int sm_count = 0;
  int smem_optin = 0;
};

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
DeviceArrays g_arrays[kMaxDevices];

// Device addresses of the arrays for `dev` (which must be current).  In host
// code the array names are host-side stand-ins, not device addresses, so the
// addresses come from cudaGetSymbolAddress, once per device.
gbblas_status_t device_arrays(int dev, DeviceArrays** out) {
  if (dev < 0 || dev >= kMaxDevices) return gb::fail(GBBLAS_STATUS_UNSUPPORTED, "sgemv_noalloc: device index too large");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  DeviceArrays& d = g_arrays[dev];
  if (!d.ready) {
    GB_CUDA_TRY(cudaGetSymbolAddress(&d.scratch, g_noalloc_scratch));
    GB_CUDA_TRY(cudaGetSymbolAddress(reinterpret_cast<void**>(&d.tickets), g_noalloc_tickets));
    GB_CUDA_TRY(cudaGetSymbolAddress(reinterpret_cast<void**>(&d.error), g_noalloc_error));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    d.ready = true;
  }
  *out = &d;
  return GBBLAS_STATUS_SUCCESS;
}

}  // namespace

extern "C" gbblas_status_t gbblas_sgemv_noalloc(void* stream, char trans, int64_t m, int64_t n, float alpha,
                                                const float* a, int64_t lda, const float* x, int64_t incx,
                                                float beta, float* y, int64_t incy) {
  gb::clear_error();
  // the argument rules of gbblas_sgemv, checked before anything is enqueued
  if (m < 0 || n < 0) return gb::fail(GBBLAS_STATUS_INVALID_ARG, "gemv: negative dimension");
  if (incx == 0 || incy == 0) return gb::fail(GBBLAS_STATUS_INVALID_ARG, "gemv: zero increment");
  if (lda < 0) return gb::fail(GBBLAS_STATUS_INVALID_ARG, "gemv: negative lda");
  const bool tr = !(trans == 'n' || trans == 'N');
  const int64_t xlen = tr ? m : n, ylen = tr ? n : m;
  if (ylen == 0) return GBBLAS_STATUS_SUCCESS;
  if (!y || (xlen > 0 && (!a || !x))) return gb::fail(GBBLAS_STATUS_INVALID_ARG, "gemv: null pointer");
  int dev = 0, stream_dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  GB_CUDA_TRY(cudaStreamGetDevice(static_cast<cudaStream_t>(stream), &stream_dev));
  if (stream_dev != dev)
    return gb::fail(GBBLAS_STATUS_INVALID_ARG, "sgemv_noalloc: the stream belongs to another device than the current one");
  DeviceArrays* d = nullptr;
  GB_TRY(device_arrays(dev, &d));
  gbblas_handle_s h;  // lives on the stack: nothing to allocate or free
  h.stream = static_cast<cudaStream_t>(stream);
  h.device = dev;
  h.sm_count = d->sm_count;
  h.max_smem_optin = d->smem_optin;
  h.temp = d->scratch;
  h.temp_size = kNoAllocScratchBytes;
  h.tickets = d->tickets;
  h.n_tickets = gb::kMaxTickets;
  h.dev_error = d->error;
  h.no_alloc = true;
  // Tickets must start at zero.  The kernels reset the ones they use; this
  // also clears any left behind by an earlier call that gave up on the
  // device.  Each output tile holds at least one output element and takes at
  // most one ticket, so the first min(ylen, kMaxTickets) are all a call uses.
  const size_t n_clear = size_t(ylen) < gb::kMaxTickets ? size_t(ylen) : gb::kMaxTickets;
  GB_CUDA_TRY(cudaMemsetAsync(d->tickets, 0, sizeof(unsigned int) * n_clear, h.stream));
  return gbblas_sgemv(&h, trans, m, n, alpha, a, lda, x, incx, beta, y, incy);
}

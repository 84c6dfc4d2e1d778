// C ABI: the mixed workload from host buffers without allocating anything.
//
// gal_run_mixed_host copies the caller's class trace into a device buffer
// that the library cudaMallocs on first use. Some callers cannot let a call
// allocate: a serving loop that must never hit cudaMalloc's implicit device
// synchronisation in the middle of its request handling, or a process whose
// device memory is carved up up front (the rest of HBM handed to other pools)
// so that a fresh allocation at run time would fail or evict someone else.
// gal_run_mixed_host_noalloc serves them: its scratch space (the trace copy
// and the stats words) lives in a fixed array compiled into this library.
#include <cuda_runtime.h>
#include <stdint.h>

#include "capi_internal.h"

namespace {

constexpr uint64_t kStatsOffset = GAL_NOALLOC_TRACE_MAX_BYTES;  // 256-byte aligned
constexpr uint64_t kScratchBytes = GAL_NOALLOC_TRACE_MAX_BYTES + 256;

// One copy per GPU that loads this library, held until process exit. Host
// code must not use this name as a device address; it takes the address from
// cudaGetSymbolAddress below.
static __device__ __align__(256) uint8_t g_noalloc_scratch[kScratchBytes];

// Device address of the scratch array in the current device's context. It
// is looked up on every call, so a context made after cudaDeviceReset gets
// its own array's address rather than a stale one. Under CUDA's default lazy
// module loading, the first lookup on a device also loads the module that
// holds the array, which is when the driver commits its memory.
int scratch_for_current_device(uint8_t **out) {
  void *ptr = nullptr;
  GAL_CUDA_TRY(cudaGetSymbolAddress(&ptr, g_noalloc_scratch), "cudaGetSymbolAddress(noalloc scratch)");
  *out = (uint8_t *)ptr;
  return GAL_OK;
}

}  // namespace

extern "C" int gal_run_mixed_host_noalloc(gal_allocator *h, uint64_t n_threads, uint32_t rounds, uint64_t seed,
                                          uint32_t seg_every, uint64_t seg_lo, uint64_t seg_hi,
                                          const uint8_t *h_classes, uint32_t block_dim, uint64_t *h_stats,
                                          void *stream) {
  if (h == nullptr || h_classes == nullptr || h_stats == nullptr) return galcapi::fail_invalid("NULL argument");
  const uint64_t bytes = n_threads * (uint64_t)rounds;
  if (rounds != 0 && bytes / rounds != n_threads) return galcapi::fail_invalid("trace size overflows");
  if (bytes > GAL_NOALLOC_TRACE_MAX_BYTES)
    return galcapi::fail_invalid(
        "class trace larger than the 2 MiB static scratch of gal_run_mixed_host_noalloc "
        "(n_threads * rounds must be <= 2097152); use gal_run_mixed_host");
  uint8_t *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != GAL_OK) return rc;
  uint8_t *d_trace = scratch;
  unsigned long long *d_stats = (unsigned long long *)(scratch + kStatsOffset);
  cudaStream_t s = (cudaStream_t)stream;
  // the array keeps the previous call's contents: the stats must start at zero
  GAL_CUDA_TRY(cudaMemsetAsync(d_stats, 0, 8 * sizeof(unsigned long long), s), "noalloc stats reset");
  if (bytes) GAL_CUDA_TRY(cudaMemcpyAsync(d_trace, h_classes, bytes, cudaMemcpyHostToDevice, s), "noalloc trace H2D");
  rc = gal_run_mixed(h, n_threads, rounds, seed, seg_every, seg_lo, seg_hi, d_trace, block_dim, d_stats, stream);
  if (rc != GAL_OK) return rc;
  GAL_CUDA_TRY(cudaMemcpyAsync(h_stats, d_stats, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s),
               "noalloc stats D2H");
  GAL_CUDA_TRY(cudaStreamSynchronize(s), "noalloc sync");
  return GAL_OK;
}

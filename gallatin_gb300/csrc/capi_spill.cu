// C ABI: device-first allocation with a host-arena fallback (fused
// fill/drain) and the zeroed-memory check for GAL_FLAG_CALLOC allocators.
#include <cuda_runtime.h>

#include "capi_internal.h"
#include "device_alloc.cuh"
#include "spill_workloads.cuh"

namespace {

cudaStream_t as_stream(void *s) { return (cudaStream_t)s; }

constexpr unsigned kBlock = 256;

}  // namespace

using galcapi::fail_invalid;
using galcapi::grid_for;

extern "C" int gal_run_fused(gal_allocator *dev, gal_allocator *host, uint64_t n, uint64_t seed,
                             const uint8_t *d_classes, uint64_t *d_table, uint32_t phase_mask,
                             unsigned long long *d_stats, void *stream) {
  if (dev == nullptr || d_table == nullptr || d_stats == nullptr) return fail_invalid("NULL argument");
  if (host == dev) return fail_invalid("the host allocator must be a second allocator");
  if (phase_mask == 0 || (phase_mask & ~3u)) return fail_invalid("phase_mask must be 1, 2 or 3");
  if (n == 0) return GAL_OK;
  galwork::fused_alloc<gal_device_alloc> f{reinterpret_cast<gal_device_alloc *>(dev->d_state),
                                           host ? reinterpret_cast<gal_device_alloc *>(host->d_state) : nullptr};
  cudaStream_t s = as_stream(stream);
  if (phase_mask & 1u) {
    galwork::fill_kernel<gal_device_alloc><<<grid_for(n, kBlock), kBlock, 0, s>>>(f, n, seed, d_classes, d_table,
                                                                                 d_stats);
    GAL_CUDA_TRY(cudaGetLastError(), "fill launch");
  }
  if (phase_mask & 2u) {
    galwork::drain_kernel<gal_device_alloc><<<grid_for(n, kBlock), kBlock, 0, s>>>(f, n, seed, d_classes, d_table,
                                                                                  d_stats);
    GAL_CUDA_TRY(cudaGetLastError(), "drain launch");
  }
  return GAL_OK;
}

extern "C" int gal_run_fused_host(gal_allocator *dev, gal_allocator *host, uint64_t n, uint64_t seed,
                                  const uint8_t *h_classes, uint64_t *h_stats, void *stream) {
  if (dev == nullptr || h_classes == nullptr || h_stats == nullptr) return fail_invalid("NULL argument");
  // scratch owned by `dev`: the pointer table (8 B per request) followed by
  // the class trace (1 B per request), grown on demand
  const uint64_t table_bytes = n * 8, bytes = table_bytes + n;
  if (bytes > dev->d_ftable_bytes) {
    if (dev->d_ftable) cudaFree(dev->d_ftable);
    dev->d_ftable = nullptr;
    dev->d_ftable_bytes = 0;
    GAL_CUDA_TRY(cudaMalloc(&dev->d_ftable, bytes), "cudaMalloc fused scratch");
    dev->d_ftable_bytes = bytes;
  }
  uint8_t *d_classes = (uint8_t *)dev->d_ftable + table_bytes;
  cudaStream_t s = as_stream(stream);
  GAL_CUDA_TRY(cudaMemsetAsync(dev->d_stats, 0, 64, s), "stats reset");
  GAL_CUDA_TRY(cudaMemcpyAsync(d_classes, h_classes, n, cudaMemcpyHostToDevice, s), "trace H2D");
  const int rc = gal_run_fused(dev, host, n, seed, d_classes, dev->d_ftable, 3u, dev->d_stats, stream);
  if (rc != GAL_OK) return rc;
  GAL_CUDA_TRY(cudaMemcpyAsync(h_stats, dev->d_stats, 64, cudaMemcpyDeviceToHost, s), "stats D2H");
  GAL_CUDA_TRY(cudaStreamSynchronize(s), "e2e sync");
  return GAL_OK;
}

extern "C" int gal_run_zeroed(gal_allocator *h, uint64_t n_threads, uint32_t rounds, uint64_t seed,
                              uint32_t big_every, uint64_t big_lo, uint64_t big_hi, unsigned long long *d_stats,
                              void *stream) {
  if (h == nullptr || d_stats == nullptr) return fail_invalid("NULL argument");
  if (big_every && (big_lo == 0 || big_hi < big_lo)) return fail_invalid("bad large-request size range");
  if (n_threads == 0) return GAL_OK;
  galwork::zeroed_kernel<gal_device_alloc><<<grid_for(n_threads, kBlock), kBlock, 0, as_stream(stream)>>>(
      reinterpret_cast<gal_device_alloc *>(h->d_state), n_threads, rounds, seed, big_every, big_lo, big_hi, d_stats);
  GAL_CUDA_TRY(cudaGetLastError(), "zeroed launch");
  return GAL_OK;
}

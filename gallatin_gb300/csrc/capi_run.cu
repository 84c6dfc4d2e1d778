// C ABI: batch malloc/free, pinned-block flush, and the benchmark workloads,
// all launched over the device allocator inlined from alloc.cuh.
#include <cuda_runtime.h>

#include "capi_internal.h"
#include "device_alloc.cuh"
#include "workloads.cuh"

namespace {

__global__ void malloc_batch_kernel(const gal_state_t *st, const uint64_t *sizes, uint64_t n, uint64_t *out) {
  const uint64_t tid = (uint64_t)threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  out[tid] = (uint64_t)gal::malloc(st, sizes[tid]);
}

__global__ void free_batch_kernel(const gal_state_t *st, const uint64_t *ptrs, uint64_t n) {
  const uint64_t tid = (uint64_t)threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  gal::free(st, (void *)ptrs[tid]);
}

__global__ void flush_kernel(const gal_state_t *st, uint32_t total_slots) {
  const uint32_t tid = threadIdx.x + blockIdx.x * blockDim.x;
  if (tid >= total_slots) return;
  gal::flush_slot(st, st->slots + tid);
}

// Device size classing of each request: the dispatch malloc applies and the
// bytes the request really occupies.
__global__ void size_classes_kernel(const gal_state_t *st, const uint64_t *sizes, uint64_t n, gal_size_info_t *out) {
  const uint64_t tid = (uint64_t)threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  const uint64_t size = sizes[tid];
  const gal::size_class sc = gal::classify(st, size);
  gal_size_info_t r;
  r.tier = (uint32_t)sc.tier;
  r.tree = sc.tree;
  r.count = sc.tier == gal::TIER_SEGMENT ? sc.nseg : sc.count;
  r.allocated = gal::allocated_size(st, size);
  out[tid] = r;
}

// L2 atomic throughput probe. Lane 0 of every warp issues kProbeInFlight
// independent 64-bit atomic adds per iteration, each to its own 128-byte
// line, the way the allocator's group leaders touch block words; mode 0
// returns the old value (atom), mode 1 does not (red). `lines` is a power
// of two; warp w, iteration i, slot k uses line (w + (i * kProbeInFlight +
// k) * nwarps) mod lines, so concurrent warps never share a line.
constexpr uint32_t kProbeInFlight = 8;

__global__ void l2_atomic_probe_kernel(uint64_t *words, uint64_t lines, uint32_t iters, uint32_t mode,
                                       unsigned long long *sink) {
  const uint64_t gtid = (uint64_t)threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if ((threadIdx.x & 31) != 0) return;
  const uint64_t warp = gtid >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t mask = lines - 1;
  uint64_t acc = 0;
  for (uint32_t it = 0; it < iters; ++it) {
    uint64_t v[kProbeInFlight];
#pragma unroll
    for (uint32_t k = 0; k < kProbeInFlight; ++k) {
      uint64_t *p = words + (((warp + ((uint64_t)it * kProbeInFlight + k) * nwarps) & mask) << 4);
      if (mode == 0) {
        v[k] = gal::ptx::atom_add_relaxed(p, 1);
      } else {
        gal::ptx::red_add_relaxed(p, 1);
        v[k] = 0;
      }
    }
#pragma unroll
    for (uint32_t k = 0; k < kProbeInFlight; ++k) acc += v[k];
  }
  if (acc == 0x5A5A5A5A5A5A5A5Aull) *sink = acc;  // keeps the returned values live
}

cudaStream_t as_stream(void *s) { return (cudaStream_t)s; }

}  // namespace

using galcapi::fail_invalid;
using galcapi::grid_for;

extern "C" int gal_malloc_batch(gal_allocator *h, const uint64_t *d_sizes, uint64_t n, uint64_t *d_ptrs,
                                void *stream) {
  if (h == nullptr || (n && (d_sizes == nullptr || d_ptrs == nullptr))) return fail_invalid("NULL argument");
  if (n == 0) return GAL_OK;
  malloc_batch_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(h->d_state, d_sizes, n, d_ptrs);
  GAL_CUDA_TRY(cudaGetLastError(), "malloc_batch launch");
  return GAL_OK;
}

extern "C" int gal_free_batch(gal_allocator *h, const uint64_t *d_ptrs, uint64_t n, void *stream) {
  if (h == nullptr || (n && d_ptrs == nullptr)) return fail_invalid("NULL argument");
  if (n == 0) return GAL_OK;
  free_batch_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(h->d_state, d_ptrs, n);
  GAL_CUDA_TRY(cudaGetLastError(), "free_batch launch");
  return GAL_OK;
}

extern "C" int gal_size_classes(gal_allocator *h, const uint64_t *d_sizes, uint64_t n, gal_size_info_t *d_out,
                                void *stream) {
  if (h == nullptr || (n && (d_sizes == nullptr || d_out == nullptr))) return fail_invalid("NULL argument");
  if (n == 0) return GAL_OK;
  size_classes_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(h->d_state, d_sizes, n, d_out);
  GAL_CUDA_TRY(cudaGetLastError(), "size_classes launch");
  return GAL_OK;
}

extern "C" int gal_probe_l2_atomics(uint64_t *d_words, uint64_t lines, uint32_t iters, uint32_t mode,
                                    uint32_t ctas_per_sm, unsigned long long *d_sink, uint64_t *ops_out,
                                    void *stream) {
  if (d_words == nullptr || d_sink == nullptr || ops_out == nullptr) return fail_invalid("NULL argument");
  if (lines == 0 || (lines & (lines - 1)) != 0) return fail_invalid("lines must be a power of two");
  if (mode > 1 || ctas_per_sm == 0 || ctas_per_sm > 8) return fail_invalid("bad probe mode or geometry");
  int dev = 0, sms = 0;
  GAL_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  GAL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  const uint32_t grid = (uint32_t)sms * ctas_per_sm;
  const uint64_t nwarps = (uint64_t)grid * 256 / 32;
  if (nwarps > lines) return fail_invalid("fewer lines than warps: warps would share lines");
  l2_atomic_probe_kernel<<<grid, 256, 0, as_stream(stream)>>>(d_words, lines, iters, mode, d_sink);
  GAL_CUDA_TRY(cudaGetLastError(), "l2 atomic probe launch");
  *ops_out = nwarps * (uint64_t)iters * kProbeInFlight;
  return GAL_OK;
}

extern "C" int gal_flush_pinned(gal_allocator *h, void *stream) {
  if (h == nullptr) return fail_invalid("handle is NULL");
  const uint32_t total = h->hs.total_slots;
  flush_kernel<<<grid_for(total, 128), 128, 0, as_stream(stream)>>>(h->d_state, total);
  GAL_CUDA_TRY(cudaGetLastError(), "flush launch");
  GAL_CUDA_TRY(cudaMemsetAsync(h->hs.nomem, 0, sizeof(uint32_t), as_stream(stream)), "nomem reset");
  return GAL_OK;
}

extern "C" int gal_run_pairs(gal_allocator *h, uint64_t n_threads, uint64_t size, uint32_t block_dim,
                             unsigned long long *d_stats, void *stream) {
  if (h == nullptr || d_stats == nullptr) return fail_invalid("NULL argument");
  if (block_dim == 0 || block_dim > 1024 || block_dim % 32) return fail_invalid("block_dim must be 32..1024, x32");
  if (n_threads == 0) return GAL_OK;
  // compiled for two CTAs of 1024 threads per SM: 11 % faster on the 16 B
  // configuration than one, although the malloc path spills at 32 registers
  galwork::pairs_kernel<gal_device_alloc, 2><<<grid_for(n_threads, block_dim), block_dim, 0, as_stream(stream)>>>(
      reinterpret_cast<gal_device_alloc *>(h->d_state), n_threads, size, d_stats);
  GAL_CUDA_TRY(cudaGetLastError(), "pairs launch");
  return GAL_OK;
}

extern "C" int gal_run_mixed(gal_allocator *h, uint64_t n_threads, uint32_t rounds, uint64_t seed,
                             uint32_t seg_every, uint64_t seg_lo, uint64_t seg_hi, const uint8_t *d_classes,
                             uint32_t block_dim, unsigned long long *d_stats, void *stream) {
  if (h == nullptr || d_stats == nullptr) return fail_invalid("NULL argument");
  if (block_dim == 0 || block_dim > 1024 || block_dim % 32) return fail_invalid("block_dim must be 32..1024, x32");
  if (seg_every && (seg_lo == 0 || seg_hi < seg_lo)) return fail_invalid("bad segment-tier size range");
  if (n_threads == 0) return GAL_OK;
  galwork::mixed_kernel<gal_device_alloc><<<grid_for(n_threads, block_dim), block_dim, 0, as_stream(stream)>>>(
      reinterpret_cast<gal_device_alloc *>(h->d_state), n_threads, rounds, seed, seg_every, seg_lo, seg_hi, d_classes,
      d_stats);
  GAL_CUDA_TRY(cudaGetLastError(), "mixed launch");
  return GAL_OK;
}

extern "C" int gal_run_mixed_host(gal_allocator *h, uint64_t n_threads, uint32_t rounds, uint64_t seed,
                                  uint32_t seg_every, uint64_t seg_lo, uint64_t seg_hi, const uint8_t *h_classes,
                                  uint32_t block_dim, uint64_t *h_stats, void *stream) {
  if (h == nullptr || h_classes == nullptr || h_stats == nullptr) return fail_invalid("NULL argument");
  const uint64_t bytes = n_threads * (uint64_t)rounds;
  if (bytes > h->d_classes_bytes) {
    if (h->d_classes) cudaFree(h->d_classes);
    h->d_classes = nullptr;
    h->d_classes_bytes = 0;
    GAL_CUDA_TRY(cudaMalloc(&h->d_classes, bytes), "cudaMalloc class trace");
    h->d_classes_bytes = bytes;
  }
  cudaStream_t s = as_stream(stream);
  GAL_CUDA_TRY(cudaMemsetAsync(h->d_stats, 0, 64, s), "stats reset");
  GAL_CUDA_TRY(cudaMemcpyAsync(h->d_classes, h_classes, bytes, cudaMemcpyHostToDevice, s), "trace H2D");
  int rc = gal_run_mixed(h, n_threads, rounds, seed, seg_every, seg_lo, seg_hi, h->d_classes, block_dim,
                         h->d_stats, stream);
  if (rc != GAL_OK) return rc;
  GAL_CUDA_TRY(cudaMemcpyAsync(h_stats, h->d_stats, 64, cudaMemcpyDeviceToHost, s), "stats D2H");
  GAL_CUDA_TRY(cudaStreamSynchronize(s), "e2e sync");
  return GAL_OK;
}

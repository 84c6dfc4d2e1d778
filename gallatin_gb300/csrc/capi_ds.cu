// C ABI: the allocator-backed chained hash table and the vector-growth run
// (gallatin_gb300/structures.cuh, ds_workloads.cuh) over this allocator.
#include <cuda_runtime.h>

#include "capi_internal.h"
#include "device_alloc.cuh"
#include "ds_workloads.cuh"

struct gal_table {
  gal_allocator *owner;
  galds::chaining_table<gal_device_alloc> t;
};

namespace {

constexpr unsigned kBlock = 256;

__global__ void chain_stats_kernel(galds::chaining_table<gal_device_alloc> t, unsigned long long *out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned len = i < t.nbuckets ? t.chain_length(i) : 0;
  const unsigned mx = __reduce_max_sync(0xffffffffu, len);
  const unsigned sum = __reduce_add_sync(0xffffffffu, len);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, (unsigned long long)mx);
    atomicAdd(out + 1, (unsigned long long)sum);
  }
}

}  // namespace

extern "C" int gal_table_create(gal_allocator *h, uint64_t nbuckets, uint64_t seed, gal_table **out) {
  if (out == nullptr) return galcapi::fail_invalid("out is NULL");
  *out = nullptr;
  if (h == nullptr) return galcapi::fail_invalid("handle is NULL");
  if (nbuckets == 0) return galcapi::fail_invalid("nbuckets must be positive");
  gal_table *tb = new gal_table();
  tb->owner = h;
  tb->t.alloc = reinterpret_cast<gal_device_alloc *>(h->d_state);
  tb->t.nbuckets = nbuckets;
  tb->t.seed = seed;
  tb->t.heads = nullptr;
  cudaError_t e = cudaMalloc(&tb->t.heads, nbuckets * sizeof(void *));
  if (e == cudaSuccess) e = cudaMemset(tb->t.heads, 0, nbuckets * sizeof(void *));
  if (e != cudaSuccess) {
    if (tb->t.heads) cudaFree(tb->t.heads);
    delete tb;
    return galcapi::fail_cuda(e, "table directory");
  }
  *out = tb;
  return GAL_OK;
}

extern "C" int gal_table_op(gal_table *tb, uint32_t op, const uint64_t *d_keys, uint64_t n, uint64_t key_seed,
                            unsigned long long *d_stats, void *stream) {
  if (tb == nullptr || d_stats == nullptr) return galcapi::fail_invalid("NULL argument");
  if (op > GAL_TABLE_QUERY_AFTER_ERASE) return galcapi::fail_invalid("unknown table op");
  const bool per_bucket = op == GAL_TABLE_COMPACT || op == GAL_TABLE_CLEAR;
  const uint64_t items = per_bucket ? tb->t.nbuckets : n;
  if (items == 0) return GAL_OK;
  galdswork::launch_table_op(tb->t, d_keys, n, key_seed, op, d_stats, items, kBlock, (cudaStream_t)stream);
  GAL_CUDA_TRY(cudaGetLastError(), "table launch");
  return GAL_OK;
}

extern "C" int gal_table_chain_stats(gal_table *tb, uint64_t *max_len, uint64_t *total_nodes) {
  if (tb == nullptr || max_len == nullptr || total_nodes == nullptr) return galcapi::fail_invalid("NULL argument");
  unsigned long long *d = nullptr;
  GAL_CUDA_TRY(cudaMalloc(&d, 16), "chain stats scratch");
  cudaMemset(d, 0, 16);
  chain_stats_kernel<<<galcapi::grid_for(tb->t.nbuckets, kBlock), kBlock>>>(tb->t, d);
  unsigned long long hst[2] = {0, 0};
  cudaError_t e = cudaMemcpy(hst, d, 16, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return galcapi::fail_cuda(e, "chain stats");
  *max_len = hst[0];
  *total_nodes = hst[1];
  return GAL_OK;
}

extern "C" int gal_table_destroy(gal_table *tb) {
  if (tb == nullptr) return GAL_OK;
  GAL_CUDA_TRY(cudaDeviceSynchronize(), "table destroy sync");
  cudaFree(tb->t.heads);
  delete tb;
  return GAL_OK;
}

extern "C" int gal_run_vectors(gal_allocator *h, const uint32_t *d_lengths, uint64_t n, uint32_t start,
                               unsigned long long *d_stats, void *stream) {
  if (h == nullptr || d_lengths == nullptr || d_stats == nullptr) return galcapi::fail_invalid("NULL argument");
  if (n == 0) return GAL_OK;
  galdswork::vectors_kernel<gal_device_alloc><<<galcapi::grid_for(n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<gal_device_alloc *>(h->d_state), d_lengths, n, start, d_stats);
  GAL_CUDA_TRY(cudaGetLastError(), "vectors launch");
  return GAL_OK;
}

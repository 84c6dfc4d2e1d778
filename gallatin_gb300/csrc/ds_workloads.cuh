// Workload kernels over the allocator-backed data structures
// (gallatin_gb300/structures.cuh), templated on the allocator like
// workloads.cuh so the reference's allocator runs the same code.
//
// Hash table: keys are splitmix64(seed + i) (64M uniform u64 keys in the
// benchmark), values splitmix64(key). Key i is in the erased half when
// splitmix64(seed ^ (i * golden)) is odd.
// Vectors: vector v pushes lengths[v] items, item i = (v * 2654435761 + i)
// mod 2^32, then checks every item, then frees its backing.
#ifndef GALLATIN_GB300_DS_WORKLOADS_CUH
#define GALLATIN_GB300_DS_WORKLOADS_CUH

#include <stdint.h>

#include "gallatin_gb300/structures.cuh"
#include "workloads.cuh"

namespace galdswork {

enum { DS_FAIL = 0, DS_MISS = 1, DS_WRONG = 2, DS_NODES_FREED = 3, DS_PUSHES = 4 };
enum { OP_INSERT = 0, OP_ERASE_HALF = 1, OP_REINSERT_HALF = 2, OP_QUERY = 3, OP_COMPACT = 4, OP_CLEAR = 5,
       OP_QUERY_AFTER_ERASE = 6 };

__device__ __forceinline__ uint64_t table_key(const uint64_t *keys, uint64_t seed, uint64_t i) {
  return keys ? keys[i] : galwork::splitmix64(seed + i);
}
__device__ __forceinline__ bool erased_half(uint64_t seed, uint64_t i) {
  return galwork::splitmix64(seed ^ (i * 0x9E3779B97F4A7C15ull)) & 1;
}

// One thread per key (ops on keys) or per bucket (compact, clear). The
// operation is a template argument: each operation's kernel holds only its
// own code, so the phases that never allocate (erase, query) do not carry the
// registers and stack of the inlined malloc path (as one kernel over every
// operation, this library's instance had a 160-byte stack frame, and its
// erase phase, which stores nothing, wrote 3.7 times the reference's sectors
// to L2).
template <class A, uint32_t op>
__global__ void GALWORK_MIXED_BOUNDS table_kernel(galds::chaining_table<A> t, const uint64_t *keys, uint64_t n,
                                                  uint64_t seed, unsigned long long *stats) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long fail = 0, miss = 0, wrong = 0, freed = 0;
  if (op == OP_COMPACT || op == OP_CLEAR) {
    if (i < t.nbuckets) freed = op == OP_COMPACT ? t.compact(i) : t.clear(i);
  } else if (i < n) {
    const uint64_t key = table_key(keys, seed, i);
    const bool half = erased_half(seed, i);
    if (op == OP_INSERT || (op == OP_REINSERT_HALF && half)) {
      fail = !t.insert(key, galwork::splitmix64(key));
    } else if (op == OP_ERASE_HALF && half) {
      miss = !t.erase(key);
    } else if (op == OP_QUERY || op == OP_QUERY_AFTER_ERASE) {
      uint64_t v = 0;
      const bool found = t.query(key, v);
      const bool want = !(op == OP_QUERY_AFTER_ERASE && half);
      if (found != want) ++miss;
      else if (found && v != galwork::splitmix64(key)) ++wrong;
    }
  }
  const uint32_t lane = threadIdx.x & 31;
  fail = __reduce_add_sync(0xffffffffu, (unsigned)fail);
  miss = __reduce_add_sync(0xffffffffu, (unsigned)miss);
  wrong = __reduce_add_sync(0xffffffffu, (unsigned)wrong);
  freed = __reduce_add_sync(0xffffffffu, (unsigned)freed);
  if (lane == 0) {
    if (fail) atomicAdd(stats + DS_FAIL, fail);
    if (miss) atomicAdd(stats + DS_MISS, miss);
    if (wrong) atomicAdd(stats + DS_WRONG, wrong);
    if (freed) atomicAdd(stats + DS_NODES_FREED, freed);
  }
}

// Launch table operation `op` over `items` threads (keys, or buckets for
// compact and clear).
template <class A>
inline void launch_table_op(const galds::chaining_table<A> &t, const uint64_t *keys, uint64_t n, uint64_t seed,
                            uint32_t op, unsigned long long *stats, uint64_t items, unsigned block, cudaStream_t s) {
  const unsigned grid = (unsigned)((items + block - 1) / block);
  switch (op) {
    case OP_INSERT: table_kernel<A, OP_INSERT><<<grid, block, 0, s>>>(t, keys, n, seed, stats); break;
    case OP_ERASE_HALF: table_kernel<A, OP_ERASE_HALF><<<grid, block, 0, s>>>(t, keys, n, seed, stats); break;
    case OP_REINSERT_HALF: table_kernel<A, OP_REINSERT_HALF><<<grid, block, 0, s>>>(t, keys, n, seed, stats); break;
    case OP_QUERY: table_kernel<A, OP_QUERY><<<grid, block, 0, s>>>(t, keys, n, seed, stats); break;
    case OP_COMPACT: table_kernel<A, OP_COMPACT><<<grid, block, 0, s>>>(t, keys, n, seed, stats); break;
    case OP_CLEAR: table_kernel<A, OP_CLEAR><<<grid, block, 0, s>>>(t, keys, n, seed, stats); break;
    default: table_kernel<A, OP_QUERY_AFTER_ERASE><<<grid, block, 0, s>>>(t, keys, n, seed, stats); break;
  }
}

__device__ __forceinline__ uint32_t vec_item(uint64_t v, uint64_t i) {
  return (uint32_t)(v * 2654435761ull + i);
}

template <class A>
__global__ void GALWORK_MIXED_BOUNDS vectors_kernel(A *a, const uint32_t *lengths, uint64_t n, uint32_t start,
                                                    unsigned long long *stats) {
  const uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long fail = 0, wrong = 0, pushes = 0;
  if (v < n) {
    galds::svector<uint32_t, A> vec;
    if (!vec.init(a, start)) {
      fail = 1;
    } else {
      const uint32_t len = lengths[v];
      for (uint32_t i = 0; i < len; ++i) {
        if (!vec.push_back(vec_item(v, i))) {
          fail = 1;
          break;
        }
        ++pushes;
      }
      for (uint64_t i = 0; i < vec.size; ++i) wrong += vec[i] != vec_item(v, i);
      vec.free_vector();
    }
  }
  const uint32_t lane = threadIdx.x & 31;
  fail = __reduce_add_sync(0xffffffffu, (unsigned)fail);
  wrong = __reduce_add_sync(0xffffffffu, (unsigned)wrong);
  pushes = __reduce_add_sync(0xffffffffu, (unsigned)pushes);
  if (lane == 0) {
    if (fail) atomicAdd(stats + DS_FAIL, fail);
    if (wrong) atomicAdd(stats + DS_WRONG, wrong);
    if (pushes) atomicAdd(stats + DS_PUSHES, pushes);
  }
}

}  // namespace galdswork

#endif  // GALLATIN_GB300_DS_WORKLOADS_CUH

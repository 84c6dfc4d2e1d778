// The device allocator seen through the malloc/free interface the workload
// templates (workloads.cuh) expect; same layout as gal_state_t.
#ifndef GALLATIN_GB300_DEVICE_ALLOC_CUH
#define GALLATIN_GB300_DEVICE_ALLOC_CUH

#include "gallatin_gb300/alloc.cuh"

struct gal_device_alloc {
  gal_state_t state;
  __device__ __forceinline__ void *malloc(uint64_t n) { return gal::malloc(&state, n); }
  __device__ __forceinline__ void free(void *p) { gal::free(&state, p); }
  __device__ __forceinline__ void *malloc_w(uint64_t n, uint32_t w) { return gal::malloc(&state, n, w); }
  __device__ __forceinline__ void free_w(void *p, uint32_t w) { gal::free(&state, p, w); }
  __device__ __forceinline__ bool owns_allocation(const void *p) const { return gal::owns_allocation(&state, p); }
  // segments not in the segment tree (formatted for a tree or part of a
  // multi-segment allocation): a snapshot, read while others may change it
  __device__ inline uint64_t owned_segments() const {
    const gal_veb_t &t = state.segment_tree;
    const unsigned long long *leaf = (const unsigned long long *)t.bits[t.num_layers - 1];
    uint64_t free_segments = 0;
    for (uint64_t w = 0; w < t.layer_words[t.num_layers - 1]; ++w) free_segments += __popcll(__ldcg(leaf + w));
    return state.num_segments - free_segments;
  }
  // the same, counted by the 32 lanes of a converged warp (all lanes get it)
  __device__ inline uint64_t owned_segments_warp(uint32_t lane) const {
    const gal_veb_t &t = state.segment_tree;
    const unsigned long long *leaf = (const unsigned long long *)t.bits[t.num_layers - 1];
    uint32_t free_segments = 0;
    for (uint64_t w = lane; w < t.layer_words[t.num_layers - 1]; w += 32) free_segments += __popcll(__ldcg(leaf + w));
    return state.num_segments - __reduce_add_sync(0xffffffffu, free_segments);
  }
};

#endif  // GALLATIN_GB300_DEVICE_ALLOC_CUH

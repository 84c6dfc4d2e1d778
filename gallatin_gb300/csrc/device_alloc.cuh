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
  // NULL at once for a slice class known to have no room (see gal::malloc_unless_full)
  __device__ __forceinline__ void *malloc_first_w(uint64_t n, uint32_t w) { return gal::malloc_unless_full(&state, n, w); }
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

// Two allocators behind one malloc/free: the device arena first, the host
// arena (GAL_FLAG_HOST_ARENA) when that returns NULL; free goes to the arena
// that owns the pointer (the reference's global_malloc_fused /
// global_free_fused, global_allocator.cuh:186-216). Lives in device memory so
// that kernels templated on the allocator type take it like the others.
struct gal_fused_device_alloc {
  gal_device_alloc *dev;
  gal_device_alloc *host;
  __device__ __forceinline__ void *malloc_w(uint64_t n, uint32_t w) {
    void *p = dev->malloc_first_w(n, w);
    return p != nullptr ? p : host->malloc_w(n, w);
  }
  __device__ __forceinline__ void free_w(void *p, uint32_t w) {
    if (dev->owns_allocation(p)) {
      dev->free_w(p, w);
    } else {
      host->free_w(p, w);
    }
  }
  __device__ __forceinline__ void *malloc(uint64_t n) { return malloc_w(n, 32); }
  __device__ __forceinline__ void free(void *p) { free_w(p, 32); }
  // segments both arenas hold, for fragmentation (both have the same segment size)
  __device__ inline uint64_t owned_segments() const { return dev->owned_segments() + host->owned_segments(); }
  __device__ inline uint64_t owned_segments_warp(uint32_t lane) const {
    return dev->owned_segments_warp(lane) + host->owned_segments_warp(lane);
  }
};

#endif  // GALLATIN_GB300_DEVICE_ALLOC_CUH

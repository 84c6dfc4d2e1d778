// Workloads for the host-arena fallback and for zeroed (calloc) allocators,
// over any allocator type with device malloc / free / owns_allocation.
//
// The fused fill/drain templates are instantiated over the GB300 allocator
// (capi_spill.cu) and over the reference's Gallatin<...>
// (the oracle/ref_*.cu harness), so both sides of the comparison run the same
// kernels.
//
//   fill   thread i: malloc 16 << class_i bytes through fused_alloc, keep the
//          pointer in table[i], write i to its first and ~i to its last u64
//   drain  thread i: check both words, free table[i] through fused_alloc,
//          clear table[i]
//          (the shape of the reference's tests/src/global_exceed_test.cu:
//          38-110, one insert kernel then one verify-and-free kernel)
//   zeroed each thread, for `rounds` rounds: malloc 16 << (x mod 12) bytes,
//          check that every byte reads zero, fill it with a non-zero
//          pattern, free it; warp 0 of every big_every-th CTA also takes one
//          allocation of a size uniform in [big_lo, big_hi] per round
//          through the same check. On an allocator that zeroes on free every
//          allocation reads zero; on one that does not, reused bytes show
//          the previous owner's pattern.
#ifndef GALLATIN_GB300_SPILL_WORKLOADS_CUH
#define GALLATIN_GB300_SPILL_WORKLOADS_CUH

#include <stdint.h>

#include "workloads.cuh"

namespace galwork {

enum { STAT_HOST = 4 };  // fill: allocations served by the host arena

// The device attempt of the pair: an allocator that can tell at once that a
// request's class has no room (malloc_first_w) skips the search.
template <class A>
__device__ __forceinline__ auto first_attempt(A *a, uint64_t n, int) -> decltype(a->malloc_first_w(n, 32u)) {
  return a->malloc_first_w(n, 32u);
}
template <class A>
__device__ __forceinline__ void *first_attempt(A *a, uint64_t n, long) {
  return a->malloc(n);
}

// Device-first allocation with a host-arena fallback over two allocators of
// one type: malloc from `dev`, and from `host` when that returns NULL; free
// to whichever arena holds the pointer. The reference's global_malloc_fused
// / global_free_fused (global_allocator.cuh:186-216) over explicit allocator
// pointers rather than its two __device__ globals.
template <class A>
struct fused_alloc {
  A *dev;
  A *host;  // NULL: the device arena alone

  __device__ __forceinline__ void *malloc(uint64_t n) const {
    if (host == nullptr) return dev->malloc(n);
    void *p = first_attempt(dev, n, 0);
    return p != nullptr ? p : host->malloc(n);
  }
  __device__ __forceinline__ void free(void *p) const {
    if (host == nullptr || dev->owns_allocation(p)) {
      dev->free(p);
    } else {
      host->free(p);
    }
  }
  __device__ __forceinline__ bool on_host(void *p) const { return host != nullptr && !dev->owns_allocation(p); }
};

__device__ __forceinline__ uint64_t fill_size(uint64_t i, uint64_t seed, const uint8_t *classes) {
  if (classes != nullptr) return 16ull << classes[i];
  uint64_t s = splitmix64(seed + i);
  return 16ull << (xorshift64(s) % 9);
}

template <class A>
__global__ void __launch_bounds__(256) fill_kernel(fused_alloc<A> f, uint64_t n, uint64_t seed,
                                                   const uint8_t *classes, uint64_t *table,
                                                   unsigned long long *stats) {
  const uint64_t i = (uint64_t)threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  bool miss = false, host = false;
  if (i < n) {
    const uint64_t size = fill_size(i, seed, classes);
    uint64_t *p = (uint64_t *)f.malloc(size);
    table[i] = (uint64_t)p;
    if (p == nullptr) {
      miss = true;
    } else {
      p[0] = i;
      p[size / 8 - 1] = ~i;
      host = f.on_host(p);
    }
  }
  const uint32_t m = __ballot_sync(0xffffffffu, miss), h = __ballot_sync(0xffffffffu, host);
  if ((threadIdx.x & 31) == 0) {
    if (m) atomicAdd(stats + STAT_MISS, (unsigned long long)__popc(m));
    if (h) atomicAdd(stats + STAT_HOST, (unsigned long long)__popc(h));
  }
}

template <class A>
__global__ void __launch_bounds__(256) drain_kernel(fused_alloc<A> f, uint64_t n, uint64_t seed,
                                                    const uint8_t *classes, uint64_t *table,
                                                    unsigned long long *stats) {
  const uint64_t i = (uint64_t)threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  bool bad = false;
  if (i < n) {
    uint64_t *p = (uint64_t *)table[i];
    if (p != nullptr) {
      const uint64_t size = fill_size(i, seed, classes);
      bad = p[0] != i || p[size / 8 - 1] != ~i;
      f.free(p);
      table[i] = 0;
    }
  }
  const uint32_t b = __ballot_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(stats + STAT_BAD, (unsigned long long)__popc(b));
}

// Check that each lane's [p, p + 16 * n16) reads zero, then fill it with v
// (non-zero); the warp walks the lanes' ranges in turn with 16-byte accesses.
// Returns, on every lane, the mask of lanes whose range was not all zero.
__device__ __forceinline__ uint32_t check_zero_then_fill(ulonglong2 *p, uint64_t n16, uint64_t v, uint32_t lane) {
  uint32_t dirty = 0;
  for (uint32_t j = 0; j < 32; ++j) {
    ulonglong2 *pj = (ulonglong2 *)__shfl_sync(0xffffffffu, (unsigned long long)p, j);
    const uint64_t nj = __shfl_sync(0xffffffffu, n16, j);
    const uint64_t vj = __shfl_sync(0xffffffffu, v, j);
    if (pj == nullptr) continue;
    uint64_t seen = 0;
    for (uint64_t i = lane; i < nj; i += 32) {
      const ulonglong2 got = load_cg(pj + i);
      seen |= got.x | got.y;
    }
    for (uint64_t i = lane; i < nj; i += 32) pj[i] = make_ulonglong2(vj, vj);
    dirty |= (uint32_t)(seen != 0) << j;
  }
  return __reduce_or_sync(0xffffffffu, dirty);
}

// Launch with blockDim a multiple of 32 (whole warps). stats: [0] NULLs,
// [1] allocations that held a non-zero byte.
template <class Alloc>
__global__ void __launch_bounds__(256) zeroed_kernel(Alloc *alloc, uint64_t n, uint32_t rounds, uint64_t seed,
                                                     uint32_t big_every, uint64_t big_lo, uint64_t big_hi,
                                                     unsigned long long *stats) {
  const uint64_t tid = (uint64_t)threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  const bool active = tid < n;
  const uint32_t lane = threadIdx.x & 31;
  const bool big_warp = big_every != 0 && blockIdx.x % big_every == 0 && threadIdx.x < 32;
  uint64_t s = splitmix64(seed + tid);
  unsigned long long misses = 0, dirty = 0;
  for (uint32_t r = 0; r < rounds; ++r) {
    if (big_warp) {
      ulonglong2 *p = nullptr;
      uint64_t n16 = 0;
      if (lane == 0) {
        const uint64_t size =
            ((big_lo + splitmix64(seed + n + (uint64_t)blockIdx.x * rounds + r) % (big_hi - big_lo + 1)) + 15) & ~15ull;
        p = (ulonglong2 *)alloc->malloc(size);
        if (p == nullptr) {
          ++misses;
        } else {
          n16 = size / 16;
        }
      }
      if (check_zero_then_fill(p, n16, (tid << 8) | r | 1u, lane) & 1u) {
        if (lane == 0) ++dirty;
      }
      // the whole warp calls free (lanes other than 0 with NULL), so a
      // zeroing allocator spreads the clear over 32 lanes
      alloc->free(p);
    }
    ulonglong2 *p = nullptr;
    uint64_t n16 = 0;
    if (active) {
      const uint64_t size = 16ull << (xorshift64(s) % 12);
      p = (ulonglong2 *)alloc->malloc(size);
      if (p == nullptr) {
        ++misses;
      } else {
        n16 = size / 16;
      }
    }
    if ((check_zero_then_fill(p, n16, (tid << 8) | r | 1u, lane) >> lane) & 1u) ++dirty;
    alloc->free(p);
  }
  if (misses) atomicAdd(stats + STAT_MISS, misses);
  if (dirty) atomicAdd(stats + STAT_BAD, dirty);
}

}  // namespace galwork

#endif  // GALLATIN_GB300_SPILL_WORKLOADS_CUH

// Scoped memory operations and warp helpers used by the allocator.
//
// Everything the allocator shares between SMs goes through gpu-scope
// relaxed/acquire/release operations written as inline PTX, so the ordering
// each step relies on is explicit (the reference uses plain loads plus
// __threadfence, gallatin.cuh:881,980,1019,1029).
#ifndef GALLATIN_GB300_PTX_CUH
#define GALLATIN_GB300_PTX_CUH

#include <stdint.h>

namespace gal {
namespace ptx {

__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
// Two adjacent words (16-byte aligned) in one 128-bit load.
__device__ __forceinline__ void ld_relaxed_v2(const uint64_t *p, uint64_t &lo, uint64_t &hi) {
  asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(lo), "=l"(hi) : "l"(p) : "memory");
}
__device__ __forceinline__ uint64_t ld_acquire(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int32_t ld_relaxed(const int32_t *p) {
  int32_t v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint16_t ld_relaxed(const uint16_t *p) {
  unsigned short v;
  asm volatile("ld.relaxed.gpu.global.u16 %0, [%1];" : "=h"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint64_t *p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_release(uint64_t *p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t atom_add_acquire(uint64_t *p, uint64_t v) {
  uint64_t r;
  asm volatile("atom.acquire.gpu.global.add.u64 %0, [%1], %2;" : "=l"(r) : "l"(p), "l"(v) : "memory");
  return r;
}
__device__ __forceinline__ uint64_t atom_add_release(uint64_t *p, uint64_t v) {
  uint64_t r;
  asm volatile("atom.release.gpu.global.add.u64 %0, [%1], %2;" : "=l"(r) : "l"(p), "l"(v) : "memory");
  return r;
}
__device__ __forceinline__ uint64_t atom_add_relaxed(uint64_t *p, uint64_t v) {
  uint64_t r;
  asm volatile("atom.relaxed.gpu.global.add.u64 %0, [%1], %2;" : "=l"(r) : "l"(p), "l"(v) : "memory");
  return r;
}
__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
// Drop the 128-byte line at p (128-byte aligned) from L2 without writing it
// back: its bytes become indeterminate until written again.
__device__ __forceinline__ void discard_l2(const void *p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}
__device__ __forceinline__ uint64_t atom_and_acquire(uint64_t *p, uint64_t v) {
  uint64_t r;
  asm volatile("atom.acquire.gpu.global.and.b64 %0, [%1], %2;" : "=l"(r) : "l"(p), "l"(v) : "memory");
  return r;
}
__device__ __forceinline__ uint64_t atom_and_relaxed(uint64_t *p, uint64_t v) {
  uint64_t r;
  asm volatile("atom.relaxed.gpu.global.and.b64 %0, [%1], %2;" : "=l"(r) : "l"(p), "l"(v) : "memory");
  return r;
}
__device__ __forceinline__ uint64_t atom_or_relaxed(uint64_t *p, uint64_t v) {
  uint64_t r;
  asm volatile("atom.relaxed.gpu.global.or.b64 %0, [%1], %2;" : "=l"(r) : "l"(p), "l"(v) : "memory");
  return r;
}
__device__ __forceinline__ void red_or_release(uint64_t *p, uint64_t v) {
  asm volatile("red.release.gpu.global.or.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_or_relaxed(uint64_t *p, uint64_t v) {
  asm volatile("red.relaxed.gpu.global.or.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_add_relaxed(uint64_t *p, uint64_t v) {
  asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_and_relaxed(uint64_t *p, uint64_t v) {
  asm volatile("red.relaxed.gpu.global.and.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t cas_acq_rel(uint64_t *p, uint64_t cmp, uint64_t v) {
  uint64_t r;
  asm volatile("atom.acq_rel.gpu.global.cas.b64 %0, [%1], %2, %3;"
               : "=l"(r) : "l"(p), "l"(cmp), "l"(v) : "memory");
  return r;
}
__device__ __forceinline__ int32_t atom_add_acquire(int32_t *p, int32_t v) {
  int32_t r;
  asm volatile("atom.acquire.gpu.global.add.s32 %0, [%1], %2;" : "=r"(r) : "l"(p), "r"(v) : "memory");
  return r;
}
__device__ __forceinline__ int32_t atom_add_release(int32_t *p, int32_t v) {
  int32_t r;
  asm volatile("atom.release.gpu.global.add.s32 %0, [%1], %2;" : "=r"(r) : "l"(p), "r"(v) : "memory");
  return r;
}
__device__ __forceinline__ int32_t cas_acq_rel(int32_t *p, int32_t cmp, int32_t v) {
  int32_t r;
  asm volatile("atom.acq_rel.gpu.global.cas.b32 %0, [%1], %2, %3;"
               : "=r"(r) : "l"(p), "r"(cmp), "r"(v) : "memory");
  return r;
}
__device__ __forceinline__ uint32_t smid() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t laneid() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%laneid;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t r;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(r));
  return r;
}

// 64-bit warp broadcast from `src` among the lanes of `mask`.
__device__ __forceinline__ uint64_t shfl64(uint32_t mask, uint64_t v, int src) {
  uint32_t lo = __shfl_sync(mask, (uint32_t)v, src);
  uint32_t hi = __shfl_sync(mask, (uint32_t)(v >> 32), src);
  return ((uint64_t)hi << 32) | lo;
}

// OR of a 64-bit value over the lanes of `mask`.
__device__ __forceinline__ uint64_t reduce_or64(uint32_t mask, uint64_t v) {
  uint32_t lo = __reduce_or_sync(mask, (uint32_t)v);
  uint32_t hi = __reduce_or_sync(mask, (uint32_t)(v >> 32));
  return ((uint64_t)hi << 32) | lo;
}

// Position of the j-th (0-based) set bit of x; x must have more than j bits.
__device__ __forceinline__ int nth_set_bit(uint64_t x, int j) {
  uint32_t lo = (uint32_t)x;
  int plo = __popc(lo);
  if (j < plo) return __fns(lo, 0, j + 1);
  return 32 + __fns((uint32_t)(x >> 32), 0, j - plo + 1);
}

}  // namespace ptx
}  // namespace gal

#endif  // GALLATIN_GB300_PTX_CUH

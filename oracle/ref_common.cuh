// ORACLE — test and baseline infrastructure only; never part of the product.
//
// Shared part of the C-ABI harness over the UNMODIFIED reference headers
// (saltsystemslab/gallatin include/gallatin/allocators/*.cuh), staged by
// oracle/build.py in oracle/_ref/include. The harness is split by workload
// family into translation units (ref_core.cu, ref_batches.cu,
// ref_serving.cu, ref_ds.cu, ref_fused.cu), each built into a library of its
// own (oracle/_ref/libgalref_<family>.so) so that they compile in parallel;
// a handle made by ref_core's galref_create is a plain struct of device
// pointers that every family's entry points accept.
#ifndef GALLATIN_GB300_ORACLE_REF_COMMON_CUH
#define GALLATIN_GB300_ORACLE_REF_COMMON_CUH

#include <gallatin/allocators/gallatin.cuh>

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "gallatin_gb300.h"  // gal_veb_op layout, op codes and serving structs only

namespace galref {

using namespace gallatin::allocators;

// the reference geometries the harness instantiates
using ref_16m_16_4096 = Gallatin<16ULL * 1024 * 1024, 16ULL, 4096ULL>;
using ref_16m_128_4096 = Gallatin<16ULL * 1024 * 1024, 128ULL, 4096ULL>;

// Host handle of one reference allocator. The layout is shared by every
// family library: keep it plain.
struct RefAlloc {
  int config;  // index into the geometries above
  void *dev;   // the reference's device pointer (Gallatin<...>*)
  uint8_t *d_classes;
  uint64_t d_classes_bytes;
  unsigned long long *d_stats;
  void *d_serve;
  uint64_t d_serve_bytes;
  void *d_fused;  // device copy of the fused pair for the fused serving loop
};

inline int config_of(uint64_t seg, uint64_t mn, uint64_t mx) {
  if (seg == (16ull << 20) && mn == 16 && mx == 4096) return 0;
  if (seg == (16ull << 20) && mn == 128 && mx == 4096) return 1;
  return -1;
}

// Call f(G*) with the handle's device pointer cast to its geometry's type.
// Each workload family is instantiated only for the geometries its callers
// use (every template instance is a full copy of the reference allocator):
// the default one, and for the table and vectors also the 128 B minimum.
// Other geometries return 1 (unsupported).
template <class F>
int with_default(RefAlloc *a, F &&f) {
  return a->config == 0 ? f((ref_16m_16_4096 *)a->dev) : 1;
}

template <class F>
int with_default_or_128(RefAlloc *a, F &&f) {
  switch (a->config) {
    case 0: return f((ref_16m_16_4096 *)a->dev);
    case 1: return f((ref_16m_128_4096 *)a->dev);
    default: return 1;
  }
}

inline int launch_status() { return cudaGetLastError() == cudaSuccess ? 0 : 2; }

}  // namespace galref

#endif  // GALLATIN_GB300_ORACLE_REF_COMMON_CUH

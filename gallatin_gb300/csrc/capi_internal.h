// Host-side definitions shared by the C-ABI translation units.
#ifndef GALLATIN_GB300_CAPI_INTERNAL_H
#define GALLATIN_GB300_CAPI_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "gallatin_gb300.h"

struct gal_allocator {
  gal_state_t hs;         // host copy; pointers are device addresses
  gal_state_t *d_state;   // device copy user kernels receive
  uint64_t min_size;
  uint64_t max_size;
  std::vector<void *> device_allocs;
  // scratch for the host-buffer entry points, grown on demand
  uint8_t *d_classes;
  uint64_t d_classes_bytes;
  unsigned long long *d_stats;
  // scratch of the host-buffer batch entry point, grown on demand
  uint64_t *d_breqs;
  uint64_t d_breqs_bytes;
  uint64_t *d_boffs;
  uint64_t d_boffs_bytes;
  uint64_t *d_btable;
  uint64_t d_btable_bytes;
  // the host-buffer batch path's copy stream and event (made on first use):
  // batch b's requests are copied while earlier batches run
  cudaStream_t copy_stream;
  cudaEvent_t copy_event;
  // scratch of the binned batch path: one sorted batch, bin counters
  uint64_t *d_bsorted;
  uint64_t d_bsorted_bytes;
  uint32_t *d_bbins;
  uint64_t d_bbins_bytes;
  // scratch of the serving loop: slot and page tables
  void *d_serve;
  uint64_t d_serve_bytes;
  // scratch of the host-buffer fused fill/drain: class trace and pointer table
  uint64_t *d_ftable;
  uint64_t d_ftable_bytes;
  // GAL_FLAG_HOST_ARENA: the pinned host allocation behind hs.memory
  char *host_arena;
  // the device-side pair (this allocator, a host-arena one) of the fused
  // serving loop, written before each such run
  void *d_fused;
};

struct gal_veb {
  gal_veb_t hv;
  gal_veb_t *d_veb;
  std::vector<void *> device_allocs;
};

namespace galcapi {

// Record a failed CUDA call; returns GAL_ERR_CUDA (or GAL_ERR_NOMEM for
// allocation failures) so callers can `return fail(...)`.
int fail_cuda(cudaError_t e, const char *what);
int fail_invalid(const char *what);
void set_error(const char *msg);

// Build vEB layers on the device; `full` sets every id < universe.
int build_veb(gal_veb_t *t, uint64_t universe, uint64_t seed, bool full, std::vector<void *> &allocs);

inline unsigned grid_for(uint64_t n, unsigned block) { return (unsigned)((n + block - 1) / block); }

}  // namespace galcapi

#define GAL_CUDA_TRY(call, what)                        \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return galcapi::fail_cuda(e_, what); \
  } while (0)

#endif  // GALLATIN_GB300_CAPI_INTERNAL_H

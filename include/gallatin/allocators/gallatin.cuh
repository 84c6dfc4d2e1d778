// Drop-in replacement for the reference's gallatin/allocators/gallatin.cuh.
//
// Same template, namespace and member names as
// gallatin::allocators::Gallatin<bytes_per_segment, smallest, biggest>
// (reference gallatin.cuh:292-2035): a host static generate_on_device that
// returns a device pointer, free_on_device, and device malloc/free that any
// thread of a user kernel may call. The device part is inlined from
// gallatin_gb300/alloc.cuh; the host part calls the C ABI in
// libgallatin_gb300.so (gallatin_gb300.h), so code that includes this header
// links against that library.
//
// Differences a user can see:
//   * running_calloc zeroes on free inside the freeing warp (every lane that
//     frees stores 16 B per step over each lane's allocation in turn) rather
//     than in child grids launched through dynamic parallelism (reference
//     gallatin.cuh:1306-1369); every tier is zeroed, slices included (the
//     reference's block clear returns blocks without writing them,
//     memory_table.cuh:101-136). A lone thread freeing a large allocation
//     clears it alone: call free from the whole warp (other lanes may pass
//     NULL) to share the work;
//   * without running_calloc the arena is not zero-filled at creation (the
//     reference memsets it, memory_table.cuh:518); like malloc, contents
//     start undefined;
//   * the geometry must satisfy biggest >= 32 * smallest.
#ifndef GALLATIN_ALLOCATORS_GALLATIN_CUH
#define GALLATIN_ALLOCATORS_GALLATIN_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../gallatin_gb300.h"
#include "../../gallatin_gb300/alloc.cuh"

namespace gallatin {
namespace allocators {

template <uint64_t bytes_per_segment, uint64_t smallest, uint64_t biggest>
struct Gallatin {
  using my_type = Gallatin<bytes_per_segment, smallest, biggest>;

  static_assert(bytes_per_segment >= biggest * 4096, "segment must hold a block of the largest slices");
  static_assert((bytes_per_segment & (bytes_per_segment - 1)) == 0, "segment size must be a power of two");
  static_assert((smallest & (smallest - 1)) == 0 && (biggest & (biggest - 1)) == 0,
                "slice sizes must be powers of two");
  static_assert(biggest >= 32 * smallest, "biggest must be at least 32 * smallest");

  // Instances live only in device memory; this is their layout.
  gal_state_t state;

  static __host__ my_type *generate_on_device(uint64_t max_bytes, uint64_t seed, bool print_info = true,
                                              bool running_calloc = false) {
    return generate(max_bytes, seed, print_info, running_calloc ? GAL_FLAG_CALLOC : 0u);
  }

  // The same allocator over pinned host memory mapped into the GPU (the
  // reference's generate_on_device_host, gallatin.cuh:423-526): the arena
  // lives in host memory, the metadata in HBM.
  static __host__ my_type *generate_on_device_host(uint64_t max_bytes, uint64_t seed, bool print_info = true,
                                                   bool running_calloc = false) {
    return generate(max_bytes, seed, print_info, GAL_FLAG_HOST_ARENA | (running_calloc ? GAL_FLAG_CALLOC : 0u));
  }

  static __host__ my_type *generate(uint64_t max_bytes, uint64_t seed, bool print_info, uint32_t flags) {
    gal_allocator *h = nullptr;
    const int rc = gal_create_ex(max_bytes, seed, bytes_per_segment, smallest, biggest, 0, flags, &h);
    if (rc != GAL_OK) {
      fprintf(stderr, "Gallatin: generate_on_device failed (%d): %s\n", rc, gal_last_error());
      return nullptr;
    }
    if (print_info) {
      gal_geometry_t g;
      gal_geometry(h, &g);
      printf("Booted Gallatin with %u trees in range %llu-%llu and %f GB of %s memory %llu segments\n", g.num_trees,
             (unsigned long long)smallest, (unsigned long long)biggest, 1.0 * max_bytes / 1024 / 1024 / 1024,
             (flags & GAL_FLAG_HOST_ARENA) ? "pinned host" : "device", (unsigned long long)g.num_segments);
    }
    return reinterpret_cast<my_type *>(gal_device_state(h));
  }

  static __host__ void free_on_device(my_type *dev_version) {
    gal_allocator *h = gal_from_device_state(dev_version);
    if (h) gal_destroy(h);
  }

  static __host__ __device__ int get_num_trees() {
    return gal::ceil_log2(biggest) - gal::ceil_log2(smallest) + 1;
  }

  static __host__ __device__ uint64_t get_blocks_per_segment(uint16_t tree) {
    return bytes_per_segment / ((smallest << tree) * 4096);
  }

  static __host__ __device__ uint64_t get_max_allocations_per_segment() { return bytes_per_segment / smallest; }

  __device__ void *malloc(uint64_t size) { return gal::malloc(&state, size); }

  __device__ void free(void *allocation) { gal::free(&state, allocation); }

  // malloc that returns NULL at once for a slice class whose last block
  // replacement found the arena out of blocks (no reference counterpart;
  // the fused calls use it before falling back to host memory)
  __device__ void *malloc_unless_full(uint64_t size) { return gal::malloc_unless_full(&state, size); }

  __device__ uint64_t get_allocated_size(uint64_t bytes_needed) { return gal::allocated_size(&state, bytes_needed); }

  __device__ bool owns_allocation(void *alloc) { return gal::owns_allocation(&state, alloc); }

  // Called on the device pointer from host code, like the reference.
  __host__ void print_info() {
    gal_allocator *h = gal_from_device_state(this);
    if (h) gal_print_info(h);
  }
};

}  // namespace allocators
}  // namespace gallatin

#endif  // GALLATIN_ALLOCATORS_GALLATIN_CUH

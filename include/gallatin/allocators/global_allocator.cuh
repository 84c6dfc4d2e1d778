// Drop-in replacement for the reference's gallatin/allocators/global_allocator.cuh
// (global_allocator.cuh:41-216): one default-typed allocator published through
// a __device__ pointer, plus free functions; a second one over pinned host
// memory (the _host functions); both together (_combined); and device-first
// allocation that falls back to the host arena (_fused). As in the
// reference, the __device__ variables are defined in this header, so include
// it from one translation unit (or compile with relocatable device code and
// include it from exactly one).
#ifndef GALLATIN_ALLOCATORS_GLOBAL_ALLOCATOR_CUH
#define GALLATIN_ALLOCATORS_GLOBAL_ALLOCATOR_CUH

#include "gallatin.cuh"

namespace gallatin {
namespace allocators {

using global_allocator_type = gallatin::allocators::Gallatin<16ULL * 1024 * 1024, 16ULL, 4096ULL>;

__device__ global_allocator_type *global_gallatin;
__device__ global_allocator_type *global_host_gallatin;

__host__ inline void init_global_allocator(uint64_t num_bytes, uint64_t seed, bool print_info = true,
                                           bool running_calloc = false) {
  global_allocator_type *local_copy =
      global_allocator_type::generate_on_device(num_bytes, seed, print_info, running_calloc);
  cudaMemcpyToSymbol(global_gallatin, &local_copy, sizeof(global_allocator_type *));
  cudaDeviceSynchronize();
}

__host__ inline void free_global_allocator() {
  global_allocator_type *local_copy = nullptr;
  cudaMemcpyFromSymbol(&local_copy, global_gallatin, sizeof(global_allocator_type *));
  cudaDeviceSynchronize();
  if (local_copy) global_allocator_type::free_on_device(local_copy);
  global_allocator_type *null_copy = nullptr;
  cudaMemcpyToSymbol(global_gallatin, &null_copy, sizeof(global_allocator_type *));
}

__device__ inline void *global_malloc(uint64_t num_bytes) { return global_gallatin->malloc(num_bytes); }

__device__ inline void global_free(void *ptr) { global_gallatin->free(ptr); }

__host__ inline void print_global_stats() {
  global_allocator_type *local_copy = nullptr;
  cudaMemcpyFromSymbol(&local_copy, global_gallatin, sizeof(global_allocator_type *));
  cudaDeviceSynchronize();
  if (local_copy) local_copy->print_info();
}

// ---- the host-memory allocator (reference global_allocator.cuh:98-151) ----

__host__ inline void init_global_allocator_host(uint64_t num_bytes, uint64_t seed, bool print_info = true,
                                                bool running_calloc = false) {
  global_allocator_type *local_copy =
      global_allocator_type::generate_on_device_host(num_bytes, seed, print_info, running_calloc);
  cudaMemcpyToSymbol(global_host_gallatin, &local_copy, sizeof(global_allocator_type *));
  cudaDeviceSynchronize();
}

__host__ inline void free_global_allocator_host() {
  global_allocator_type *local_copy = nullptr;
  cudaMemcpyFromSymbol(&local_copy, global_host_gallatin, sizeof(global_allocator_type *));
  cudaDeviceSynchronize();
  if (local_copy) global_allocator_type::free_on_device(local_copy);
  global_allocator_type *null_copy = nullptr;
  cudaMemcpyToSymbol(global_host_gallatin, &null_copy, sizeof(global_allocator_type *));
}

__device__ inline void *global_malloc_host(uint64_t num_bytes) { return global_host_gallatin->malloc(num_bytes); }

__device__ inline void global_free_host(void *ptr) { global_host_gallatin->free(ptr); }

__host__ inline void print_global_stats_host() {
  global_allocator_type *local_copy = nullptr;
  cudaMemcpyFromSymbol(&local_copy, global_host_gallatin, sizeof(global_allocator_type *));
  cudaDeviceSynchronize();
  if (local_copy) local_copy->print_info();
}

// ---- both arenas (reference global_allocator.cuh:153-183) ----

__host__ inline void init_global_allocator_combined(uint64_t num_bytes, uint64_t host_bytes, uint64_t seed,
                                                    bool print_info = true, bool running_calloc = false) {
  init_global_allocator(num_bytes, seed, print_info, running_calloc);
  init_global_allocator_host(host_bytes, seed, print_info, running_calloc);
}

__host__ inline void free_global_allocator_combined() {
  free_global_allocator();
  free_global_allocator_host();
}

__device__ inline void *global_malloc_combined(uint64_t num_bytes, bool on_host = false) {
  return on_host ? global_malloc_host(num_bytes) : global_malloc(num_bytes);
}

__device__ inline void global_free_combined(void *ptr, bool on_host = false) {
  if (on_host) {
    global_free_host(ptr);
  } else {
    global_free(ptr);
  }
}

// ---- device first, host arena when the device arena is out of room
//      (reference global_allocator.cuh:186-216); pointers stay where they
//      were placed until freed ----

__device__ inline void *global_malloc_fused(uint64_t num_bytes) {
  // a class the device arena is known to be out of goes straight to the host
  void *alloc = global_gallatin->malloc_unless_full(num_bytes);
  return alloc != nullptr ? alloc : global_malloc_host(num_bytes);
}

__device__ inline void global_free_fused(void *ptr) {
  if (global_gallatin->owns_allocation(ptr)) {
    global_free(ptr);
  } else {
    global_free_host(ptr);
  }
}

}  // namespace allocators
}  // namespace gallatin

#endif  // GALLATIN_ALLOCATORS_GLOBAL_ALLOCATOR_CUH

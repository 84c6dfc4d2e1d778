// Drop-in replacement for the reference's gallatin/allocators/global_allocator.cuh
// (global_allocator.cuh:41-97): one default-typed allocator published through
// a __device__ pointer, plus free functions. As in the reference, the
// __device__ variable is defined in this header, so include it from one
// translation unit (or compile with relocatable device code and include it
// from exactly one).
#ifndef GALLATIN_ALLOCATORS_GLOBAL_ALLOCATOR_CUH
#define GALLATIN_ALLOCATORS_GLOBAL_ALLOCATOR_CUH

#include "gallatin.cuh"

namespace gallatin {
namespace allocators {

using global_allocator_type = gallatin::allocators::Gallatin<16ULL * 1024 * 1024, 16ULL, 4096ULL>;

__device__ global_allocator_type *global_gallatin;

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

}  // namespace allocators
}  // namespace gallatin

#endif  // GALLATIN_ALLOCATORS_GLOBAL_ALLOCATOR_CUH

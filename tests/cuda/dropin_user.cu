// A user program written against the reference's public headers and API:
// it includes <gallatin/allocators/global_allocator.cuh>, so compiling it with
// -I include picks up the GB300 drop-in instead of the reference, and links
// libgallatin_gb300.so. Prints "DROPIN OK" when every check passes.
#include <gallatin/allocators/global_allocator.cuh>

#include <cstdio>

using namespace gallatin::allocators;

__global__ void global_churn(uint64_t n, int rounds, unsigned long long *errors) {
  const uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  for (int r = 0; r < rounds; ++r) {
    const uint64_t size = 16ull << ((tid + r) % 9);
    uint64_t *p = (uint64_t *)global_malloc(size);
    if (p == nullptr) {
      atomicAdd(errors, 1ull);
      continue;
    }
    p[0] = tid;
    p[size / 8 - 1] = ~tid;
    if (((volatile uint64_t *)p)[0] != tid || ((volatile uint64_t *)p)[size / 8 - 1] != ~tid) atomicAdd(errors + 1, 1ull);
    global_free(p);
  }
}

template <class Alloc>
__global__ void typed_churn(Alloc *alloc, uint64_t n, unsigned long long *errors) {
  const uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  const uint64_t size = (tid % 3 == 0) ? 128 : (tid % 3 == 1 ? 40000 : 8192);
  char *p = (char *)alloc->malloc(size);
  if (p == nullptr) {
    atomicAdd(errors, 1ull);
    return;
  }
  if (!alloc->owns_allocation(p) || alloc->get_allocated_size(size) < size) atomicAdd(errors + 1, 1ull);
  p[0] = 1;
  p[size - 1] = 2;
  alloc->free(p);
}

int main() {
  unsigned long long *errors = nullptr;
  cudaMallocManaged(&errors, 4 * sizeof(unsigned long long));
  errors[0] = errors[1] = errors[2] = errors[3] = 0;

  init_global_allocator(1ull << 30, 111, false);
  global_churn<<<(1 << 18) / 256, 256>>>(1 << 18, 4, errors);
  cudaError_t e = cudaDeviceSynchronize();
  print_global_stats();
  free_global_allocator();

  using my_alloc = Gallatin<16ull * 1024 * 1024, 128ull, 4096ull>;
  my_alloc *alloc = my_alloc::generate_on_device(512ull << 20, 7, false);
  if (alloc == nullptr) {
    printf("generate_on_device failed\n");
    return 1;
  }
  typed_churn<my_alloc><<<256, 256>>>(alloc, 65536, errors + 2);
  cudaError_t e2 = cudaDeviceSynchronize();
  alloc->print_info();
  my_alloc::free_on_device(alloc);

  printf("errors: global misses %llu verify %llu; typed misses %llu checks %llu; cuda %s %s\n", errors[0], errors[1],
         errors[2], errors[3], cudaGetErrorString(e), cudaGetErrorString(e2));
  const bool ok = e == cudaSuccess && e2 == cudaSuccess && errors[0] == 0 && errors[1] == 0 && errors[2] == 0 &&
                  errors[3] == 0;
  printf(ok ? "DROPIN OK\n" : "DROPIN FAILED\n");
  return ok ? 0 : 1;
}

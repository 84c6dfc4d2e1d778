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

// reference tests/src/gallatin_single_thread.cu shape: one thread mallocs
// n allocations in sequence, then checks and frees them in sequence
__global__ void single_thread_alloc(uint64_t n, uint64_t **table, unsigned long long *counts) {
  if (threadIdx.x + blockIdx.x * blockDim.x != 0) return;
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t size = 16ull << (i % 9);
    uint64_t *p = (uint64_t *)global_malloc(size);
    table[i] = p;
    if (p == nullptr) {
      counts[0] += 1;
      continue;
    }
    p[0] = i;
    p[size / 8 - 1] = ~i;
  }
}

__global__ void single_thread_free(uint64_t n, uint64_t **table, unsigned long long *counts) {
  if (threadIdx.x + blockIdx.x * blockDim.x != 0) return;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t *p = table[i];
    if (p == nullptr) continue;
    const uint64_t size = 16ull << (i % 9);
    if (p[0] != i || p[size / 8 - 1] != ~i) counts[1] += 1;
    global_free(p);
  }
}

// reference tests/src/global_exceed_test.cu shape: insert through the fused
// call, then verify and free through the fused call
__global__ void fused_fill(uint64_t n, uint64_t **table, unsigned long long *counts) {
  const uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  uint64_t *p = (uint64_t *)global_malloc_fused(1024);
  table[tid] = p;
  if (p == nullptr) {
    atomicAdd(counts, 1ull);
    return;
  }
  p[0] = tid;
  p[127] = ~tid;
  if (!global_gallatin->owns_allocation(p)) atomicAdd(counts + 1, 1ull);
}

__global__ void fused_drain(uint64_t n, uint64_t **table, unsigned long long *counts) {
  const uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  uint64_t *p = table[tid];
  if (p == nullptr) return;
  if (p[0] != tid || p[127] != ~tid) atomicAdd(counts + 2, 1ull);
  global_free_fused(p);
}

// every allocation of a running_calloc allocator reads zero, even after the
// previous round filled and freed the same bytes
template <class Alloc>
__global__ void calloc_rounds(Alloc *alloc, uint64_t n, int rounds, unsigned long long *dirty) {
  const uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  for (int r = 0; r < rounds; ++r) {
    const uint64_t size = 16ull << ((tid + r) % 10);
    uint64_t *p = (uint64_t *)alloc->malloc(size);
    if (p == nullptr) continue;
    uint64_t seen = 0;
    for (uint64_t i = 0; i < size / 8; ++i) seen |= ((volatile uint64_t *)p)[i];
    if (seen) atomicAdd(dirty, 1ull);
    for (uint64_t i = 0; i < size / 8; ++i) p[i] = ~0ull;
    alloc->free(p);
  }
}

template <class Alloc>
__global__ void host_arena_write(Alloc *alloc, uint64_t **out) {
  uint64_t *p = (uint64_t *)alloc->malloc(4096);
  if (p != nullptr)
    for (int i = 0; i < 512; ++i) p[i] = 0xC0FFEE00ull + i;
  *out = p;
}

int main() {
  unsigned long long *errors = nullptr;
  cudaMallocManaged(&errors, 4 * sizeof(unsigned long long));
  errors[0] = errors[1] = errors[2] = errors[3] = 0;

  init_global_allocator(1ull << 30, 111, false);
  global_churn<<<(1 << 18) / 256, 256>>>(1 << 18, 4, errors);
  cudaError_t e = cudaDeviceSynchronize();
  // one thread, 4,000 allocations in sequence, then their check and free
  uint64_t **st_table = nullptr;
  unsigned long long *st_counts = nullptr;
  cudaMalloc(&st_table, 4000 * sizeof(uint64_t *));
  cudaMallocManaged(&st_counts, 2 * sizeof(unsigned long long));
  st_counts[0] = st_counts[1] = 0;
  single_thread_alloc<<<1, 1>>>(4000, st_table, st_counts);
  single_thread_free<<<1, 1>>>(4000, st_table, st_counts);
  cudaError_t e_st = cudaDeviceSynchronize();
  cudaFree(st_table);
  print_global_stats();
  free_global_allocator();
  printf("single thread: misses %llu verify %llu; cuda %s\n", st_counts[0], st_counts[1], cudaGetErrorString(e_st));
  const bool single_ok = e_st == cudaSuccess && st_counts[0] == 0 && st_counts[1] == 0;

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

  // device arena of 4 segments, host arena of 16: 131,072 x 1 KiB (128 MiB)
  // cannot all fit on the device, so part of it lands in host memory
  init_global_allocator_combined(64ull << 20, 256ull << 20, 5, false);
  const uint64_t nf = 1 << 17;
  uint64_t **table = nullptr;
  unsigned long long *fc = nullptr;
  cudaMalloc(&table, nf * sizeof(uint64_t *));
  cudaMallocManaged(&fc, 3 * sizeof(unsigned long long));
  fc[0] = fc[1] = fc[2] = 0;
  fused_fill<<<nf / 256, 256>>>(nf, table, fc);
  fused_drain<<<nf / 256, 256>>>(nf, table, fc);
  cudaError_t e3 = cudaDeviceSynchronize();
  print_global_stats_host();
  free_global_allocator_combined();
  cudaFree(table);
  printf("fused: misses %llu on host %llu of %llu verify %llu; cuda %s\n", fc[0], fc[1],
         (unsigned long long)nf, fc[2], cudaGetErrorString(e3));
  const bool fused_ok = e3 == cudaSuccess && fc[0] == 0 && fc[2] == 0 && fc[1] > 0 && fc[1] < nf;

  // running_calloc on a device arena and on a host arena
  unsigned long long *dirty = nullptr;
  cudaMallocManaged(&dirty, 2 * sizeof(unsigned long long));
  dirty[0] = dirty[1] = 0;
  my_alloc *za = my_alloc::generate_on_device(256ull << 20, 9, false, true);
  calloc_rounds<my_alloc><<<64, 256>>>(za, 16384, 4, dirty);
  cudaError_t e4 = cudaDeviceSynchronize();
  my_alloc::free_on_device(za);
  using host_alloc = Gallatin<16ull * 1024 * 1024, 16ull, 4096ull>;
  // 16 segments: every size class of the rounds below gets segments of its own
  host_alloc *ha = host_alloc::generate_on_device_host(256ull << 20, 10, false, true);
  uint64_t **hp = nullptr;
  cudaMallocManaged(&hp, sizeof(uint64_t *));
  host_arena_write<host_alloc><<<1, 1>>>(ha, hp);
  calloc_rounds<host_alloc><<<16, 256>>>(ha, 4096, 4, dirty + 1);
  cudaError_t e5 = cudaDeviceSynchronize();
  // the host arena is host memory: the CPU reads what the kernel wrote
  bool host_read_ok = *hp != nullptr;
  for (int i = 0; host_read_ok && i < 512; ++i) host_read_ok = (*hp)[i] == 0xC0FFEE00ull + i;
  host_alloc::free_on_device(ha);
  printf("calloc: dirty device %llu host %llu; host read %s; cuda %s %s\n", dirty[0], dirty[1],
         host_read_ok ? "ok" : "bad", cudaGetErrorString(e4), cudaGetErrorString(e5));
  const bool calloc_ok = e4 == cudaSuccess && e5 == cudaSuccess && dirty[0] == 0 && dirty[1] == 0 && host_read_ok;

  printf("errors: global misses %llu verify %llu; typed misses %llu checks %llu; cuda %s %s\n", errors[0], errors[1],
         errors[2], errors[3], cudaGetErrorString(e), cudaGetErrorString(e2));
  const bool ok = e == cudaSuccess && e2 == cudaSuccess && errors[0] == 0 && errors[1] == 0 && errors[2] == 0 &&
                  errors[3] == 0 && fused_ok && calloc_ok && single_ok;
  printf(ok ? "DROPIN OK\n" : "DROPIN FAILED\n");
  return ok ? 0 : 1;
}

// Benchmark and test workloads over any allocator type with device
// malloc(uint64_t) / free(void*) members.
//
// The same templates are instantiated over the GB300 allocator (capi_run.cu)
// and over the reference's Gallatin<...> (the oracle/ref_*.cu harness), so both
// sides of a comparison run identical kernels.
//
//   pairs  each thread: p = malloc(size); store tid; read it back; free(p)
//          (the reference's per-thread correctness check,
//          tests/src/gallatin_test.cu:58-112, fused into one kernel)
//   mixed  each thread, for `rounds` rounds: size = 16 << class, where class
//          is x mod 9 of a per-thread xorshift64 seeded by splitmix64(seed +
//          tid) or read from a class trace; malloc, fill every 16 bytes with
//          (tid ^ round), verify, free. The fill and the verify are done by
//          the whole warp, one lane's allocation at a time, so each step is a
//          coalesced 512-byte access. Thread 0 of every seg_every-th CTA
//          first makes one segment-tier request of a size drawn uniformly in
//          [seg_lo, seg_hi] and touches its first and last 16 bytes.
//          Launch with blockDim a multiple of 32 (whole warps).
#ifndef GALLATIN_GB300_WORKLOADS_CUH
#define GALLATIN_GB300_WORKLOADS_CUH

#include <cooperative_groups.h>
#include <stdint.h>

// CTAs per SM the mixed workload kernel is compiled for (0: compiler's
// choice). The same value applies to every allocator the template is
// instantiated over.
#ifndef GALWORK_MIN_BLOCKS
#define GALWORK_MIN_BLOCKS 4
#endif
#if GALWORK_MIN_BLOCKS > 0
#define GALWORK_MIXED_BOUNDS __launch_bounds__(256, GALWORK_MIN_BLOCKS)
#else
#define GALWORK_MIXED_BOUNDS
#endif

namespace galwork {

enum { STAT_MISS = 0, STAT_BAD = 1, STAT_SEG_OK = 2, STAT_SEG_MISS = 3, STAT_WORDS = 8 };

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__host__ __device__ __forceinline__ uint64_t xorshift64(uint64_t &s) {
  s ^= s << 13;
  s ^= s >> 7;
  s ^= s << 17;
  return s;
}

// 16-byte load that the compiler cannot fold into the preceding stores.
__device__ __forceinline__ ulonglong2 load_cg(const ulonglong2 *p) {
  ulonglong2 v;
  asm volatile("ld.global.cg.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p));
  return v;
}

// MinBlocks: CTAs of 1024 threads per SM the kernel is compiled for (the
// register budget); each allocator's instance takes the value it runs
// fastest with.
template <class Alloc, int MinBlocks = 1>
__global__ void __launch_bounds__(1024, MinBlocks) pairs_kernel(Alloc *alloc, uint64_t n, uint64_t size,
                                                                 unsigned long long *stats) {
  const uint64_t tid = (uint64_t)threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= n) return;
  uint64_t *p = (uint64_t *)alloc->malloc(size);
  if (p == nullptr) {
    atomicAdd(stats + STAT_MISS, 1ull);
    return;
  }
  p[0] = tid;
  if (*(volatile uint64_t *)p != tid) atomicAdd(stats + STAT_BAD, 1ull);
  alloc->free(p);
}

template <class Alloc>
__global__ void GALWORK_MIXED_BOUNDS mixed_kernel(Alloc *alloc, uint64_t n, uint32_t rounds, uint64_t seed,
                                                  uint32_t seg_every, uint64_t seg_lo, uint64_t seg_hi,
                                                  const uint8_t *classes, unsigned long long *stats) {
  const uint64_t tid = (uint64_t)threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  const bool active = tid < n;
  const uint32_t lane = threadIdx.x & 31;
  if (active && seg_every != 0 && threadIdx.x == 0 && blockIdx.x % seg_every == 0) {
    const uint64_t j = blockIdx.x / seg_every;
    const uint64_t size = seg_lo + splitmix64(seed + n + j) % (seg_hi - seg_lo + 1);
    ulonglong2 *p = (ulonglong2 *)alloc->malloc(size);
    if (p != nullptr) {
      const uint64_t last = size / 16 - 1;
      p[0] = make_ulonglong2(tid, j);
      p[last] = make_ulonglong2(j, tid);
      const ulonglong2 a = load_cg(p), b = load_cg(p + last);
      if (a.x != tid || a.y != j || b.x != j || b.y != tid) atomicAdd(stats + STAT_BAD, 1ull);
      alloc->free(p);
      atomicAdd(stats + STAT_SEG_OK, 1ull);
    } else {
      atomicAdd(stats + STAT_SEG_MISS, 1ull);
    }
  }
  uint64_t s = splitmix64(seed + tid);
  unsigned long long misses = 0, bad = 0;
  for (uint32_t r = 0; r < rounds; ++r) {
    ulonglong2 *p = nullptr;
    uint64_t n16 = 0;
    const uint64_t v = tid ^ r;
    if (active) {
      const uint32_t cls = classes ? (uint32_t)classes[(uint64_t)r * n + tid] : (uint32_t)(xorshift64(s) % 9);
      const uint64_t size = 16ull << cls;
      p = (ulonglong2 *)alloc->malloc(size);
      if (p == nullptr) {
        ++misses;
      } else {
        n16 = size / 16;
      }
    }
    // The warp fills and verifies each lane's allocation in turn, 32 lanes x
    // 16 bytes per step: every byte of every allocation is written with its
    // owner's (tid ^ round) and read back from L2. Mismatches are collected
    // per buffer in a mask and reduced once, so the loads of all 32 buffers
    // can be in flight together.
    uint32_t mismatch = 0;
    for (uint32_t j = 0; j < 32; ++j) {
      ulonglong2 *pj = (ulonglong2 *)__shfl_sync(0xffffffffu, (unsigned long long)p, j);
      const uint64_t nj = __shfl_sync(0xffffffffu, n16, j);
      const uint64_t vj = __shfl_sync(0xffffffffu, v, j);
      if (pj == nullptr) continue;
      const ulonglong2 fill = make_ulonglong2(vj, vj);
      for (uint64_t i = lane; i < nj; i += 32) pj[i] = fill;
      uint64_t diff = 0;
      for (uint64_t i = lane; i < nj; i += 32) {
        const ulonglong2 got = load_cg(pj + i);
        diff |= (got.x ^ vj) | (got.y ^ vj);
      }
      mismatch |= (uint32_t)(diff != 0) << j;
    }
    if ((__reduce_or_sync(0xffffffffu, mismatch) >> lane) & 1u) ++bad;
    if (p != nullptr) alloc->free(p);
  }
  if (misses) atomicAdd(stats + STAT_MISS, misses);
  if (bad) atomicAdd(stats + STAT_BAD, bad);
}

// ---- batched request streams -------------------------------------------
//
// A request is one u64: the high 32 bits name a slot of the live-set table,
// the low 32 bits are a size. size > 0: table[slot] = malloc(size); size 0:
// free(table[slot]). The host generator only frees slots filled by an
// earlier batch, so the requests of one batch are independent.

// malloc/free with an aggregation width when the allocator offers one
template <class A>
__device__ __forceinline__ auto wl_malloc(A *a, uint64_t s, uint32_t w, int) -> decltype(a->malloc_w(s, w)) {
  return a->malloc_w(s, w);
}
template <class A>
__device__ __forceinline__ void *wl_malloc(A *a, uint64_t s, uint32_t, long) {
  return a->malloc(s);
}
template <class A>
__device__ __forceinline__ auto wl_free(A *a, void *p, uint32_t w, int) -> decltype(a->free_w(p, w)) {
  return a->free_w(p, w);
}
template <class A>
__device__ __forceinline__ void wl_free(A *a, void *p, uint32_t, long) {
  a->free(p);
}

template <class A>
__device__ __forceinline__ void serve_request(A *a, uint64_t req, uint64_t *table, uint32_t width,
                                              unsigned long long &misses) {
  const uint32_t slot = (uint32_t)(req >> 32);
  const uint32_t size = (uint32_t)req;
  if (size != 0) {
    void *p = wl_malloc(a, size, width, 0);
    if (p == nullptr) ++misses;
    table[slot] = (uint64_t)p;
  } else {
    void *p = (void *)table[slot];
    if (p != nullptr) wl_free(a, p, width, 0);  // a malloc that failed left 0
    table[slot] = 0;
  }
}

// plain path: one launch per batch, one thread per request
template <class A>
__global__ void GALWORK_MIXED_BOUNDS batch_kernel(A *a, const uint64_t *reqs, uint64_t n, uint64_t *table, uint32_t width,
                             unsigned long long *stats) {
  const uint64_t i = (uint64_t)threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  unsigned long long misses = 0;
  if (i < n) serve_request(a, reqs[i], table, width, misses);
  if (misses) atomicAdd(stats + STAT_MISS, misses);
}

// Serve requests [0, n) of one batch: each warp takes the next 32 from the
// batch's work counter (`work`, zero before the batch; one atomic per 32
// requests) until none are left. Warps that meet slow requests (a block
// replacement) take fewer, so the batch does not wait on a fixed share of a
// slow warp: on the 64-batch stream the persistent kernel took 8.5 ms this
// way and 10.5 ms with a fixed stride (larger grabs, 64 to 256 requests per
// atomic, were slower still: 10.6 to 24.8 ms). `sorted`: the requests were
// written in this launch (read past L1). Call with whole, converged warps.
template <class A>
__device__ __forceinline__ void serve_batch(A *a, const uint64_t *reqs, uint64_t n, uint32_t *work, uint64_t *table,
                                            uint32_t width, bool sorted, unsigned long long &misses) {
  const uint32_t lane = threadIdx.x & 31;
  while (true) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(work, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if ((uint64_t)base >= n) break;
    const uint64_t i = (uint64_t)base + lane;
    if (i < n) serve_request(a, sorted ? __ldcg(reqs + i) : reqs[i], table, width, misses);
  }
}

// persistent path: every batch in one cooperative launch; the grid syncs
// between batches (which also orders a batch's table writes before the next
// batch's frees read them). `work`: one counter per batch, zero at launch.
template <class A>
__global__ void GALWORK_MIXED_BOUNDS persistent_batches_kernel(A *a, const uint64_t *reqs, const uint64_t *offsets,
                                                               uint32_t n_batches, uint64_t *table, uint32_t width,
                                                               unsigned long long *stats, uint32_t *work) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  unsigned long long misses = 0;
  for (uint32_t b = 0; b < n_batches; ++b) {
    const uint64_t lo = offsets[b];
    serve_batch(a, reqs + lo, offsets[b + 1] - lo, work + b, table, width, false, misses);
    grid.sync();
  }
  if (misses) atomicAdd(stats + STAT_MISS, misses);
}

// Bin of a request for the binned path: 0 = free, else its power-of-two size
// class (16 B and below share bin 1; 2^27 B and above share bin 24).
constexpr uint32_t kBins = 25;
__device__ __forceinline__ uint32_t request_bin(uint64_t req) {
  const uint32_t size = (uint32_t)req;
  if (size == 0) return 0;
  int cl = size <= 16 ? 4 : 32 - __clz((int)(size - 1));
  if (cl > 27) cl = 27;
  return (uint32_t)(cl - 3);
}

// Binned persistent path: each batch is first counting-sorted by bin into
// `sorted` (capacity: the largest batch), so that the lanes of a warp ask for
// the same class and one reservation serves the warp. Phases per batch:
//   A  every CTA takes its bins' ranges and scatters its requests
//   B  serve the sorted batch; count the next batch's bins
// `bins` is 4 x kBins u32, zero at launch: counts and cursors, double
// buffered by batch parity. Requests are dealt to CTAs the same way in the
// count and the scatter (i = first + rank + k * threads), so the per-CTA
// counts kept in shared memory between the two phases stay valid. `work`:
// one counter per batch for the serving phase, zero at launch.
template <class A>
__global__ void GALWORK_MIXED_BOUNDS binned_batches_kernel(A *a, const uint64_t *reqs, const uint64_t *offsets,
                                                           uint32_t n_batches, uint64_t *table, uint32_t width,
                                                           unsigned long long *stats, uint64_t *sorted,
                                                           uint32_t *bins, uint32_t *work) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  __shared__ uint32_t s_cnt[kBins];
  __shared__ uint32_t s_pos[kBins];
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t rank = grid.thread_rank();
  unsigned long long misses = 0;

  auto count_batch = [&](uint32_t b) {
    uint32_t *hist = bins + (b & 1) * kBins;
    if (threadIdx.x < kBins) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t hi = offsets[b + 1];
    for (uint64_t i = offsets[b] + rank; i < hi; i += nthreads) atomicAdd(&s_cnt[request_bin(reqs[i])], 1u);
    __syncthreads();
    if (threadIdx.x < kBins && s_cnt[threadIdx.x]) atomicAdd(hist + threadIdx.x, s_cnt[threadIdx.x]);
  };

  if (n_batches) count_batch(0);
  grid.sync();
  for (uint32_t b = 0; b < n_batches; ++b) {
    uint32_t *hist = bins + (b & 1) * kBins;
    uint32_t *cursor = bins + (2 + (b & 1)) * kBins;
    // phase A: bin starts (exclusive prefix of the counts), this CTA's
    // ranges, scatter
    if (threadIdx.x == 0) {
      uint32_t run = 0;
      for (uint32_t k = 0; k < kBins; ++k) {
        const uint32_t n = __ldcg(hist + k);
        s_pos[k] = run;
        run += n;
      }
    }
    __syncthreads();
    if (threadIdx.x < kBins && s_cnt[threadIdx.x])
      s_pos[threadIdx.x] += atomicAdd(cursor + threadIdx.x, s_cnt[threadIdx.x]);
    __syncthreads();
    const uint64_t lo = offsets[b], hi = offsets[b + 1];
    for (uint64_t i = lo + rank; i < hi; i += nthreads) {
      const uint64_t req = reqs[i];
      sorted[atomicAdd(&s_pos[request_bin(req)], 1u)] = req;
    }
    grid.sync();
    // phase B: serve; recycle this parity's counters; count the next batch
    serve_batch(a, sorted, hi - lo, work + b, table, width, true, misses);
    if (blockIdx.x == 0 && threadIdx.x < kBins) {
      hist[threadIdx.x] = 0;
      cursor[threadIdx.x] = 0;
    }
    if (b + 1 < n_batches) count_batch(b + 1);
    grid.sync();
  }
  if (misses) atomicAdd(stats + STAT_MISS, misses);
}

}  // namespace galwork

#endif  // GALLATIN_GB300_WORKLOADS_CUH

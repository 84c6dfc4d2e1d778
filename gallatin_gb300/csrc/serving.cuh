// Serving loop: paged allocations for variable-length streams, admitted by
// memory, with continuous batching. Templates over the allocator type (like
// workloads.cuh) so the reference's allocator can run the plain path.
//
// A stream of L tokens takes one page (page_bytes, 16 tokens) per step until
// it holds ceil(L / 16) pages; it writes its tokens into each page, and on
// completion reads them all back into a checksum and frees its pages.
//
// Step s, phase 1: every active stream, and the k_s streams admitted at this
// step, allocates its next page (one thread each; the malloc is timed with
// %globaltimer). Phase 2: the pages of the streams that completed in phase 1
// are read back and freed, a page per thread, and their slots returned;
// thread 0 computes k_{s+1}: the
// longest arrival-ordered run of waiting streams that have arrived, fit in
// the free slots, and whose pages fit in the page budget beside the pages
// committed to admitted, unfinished streams. Admission therefore needs no
// host round trip, and streams admitted at step s overlap on the device with
// the ones already running. The persistent form runs every step in one
// cooperative launch with grid barriers between phases; the plain form
// launches each phase as its own kernel.
#ifndef GALLATIN_GB300_SERVING_CUH
#define GALLATIN_GB300_SERVING_CUH

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "workloads.cuh"

namespace galserve {

constexpr uint32_t kEmpty = 0xFFFFFFFFu;
// latency histogram: ns < 32 exact, then 32 linear buckets per octave up to
// 2^31 ns (3 % resolution)
constexpr int kHistOctaves = 26;
constexpr int kHistBuckets = 32 + kHistOctaves * 32;

__device__ __forceinline__ uint32_t hist_bucket(uint64_t ns) {
  if (ns < 32) return (uint32_t)ns;
  const int e = 63 - __clzll((long long)ns);  // >= 5
  if (e > 30) return kHistBuckets - 1;
  const uint32_t sub = (uint32_t)(ns >> (e - 5)) & 31u;
  return 32u + (uint32_t)(e - 5) * 32u + sub;
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// token `pos` of the stream with id `id`
__device__ __forceinline__ uint64_t token(uint64_t seed, uint32_t id, uint32_t pos) {
  return galwork::splitmix64(seed ^ (((uint64_t)id << 16) | pos));
}

struct trace_t {
  uint32_t n_streams;
  const uint32_t *arrivals_end;  // [steps + 1] arrivals_end[s + 1]: arrived at steps <= s
  const uint32_t *tokens;        // [n]
  const uint32_t *pages;         // [n]
  const uint64_t *page_prefix;   // [n + 1]
  const uint32_t *ids;           // [n] or null: token id of stream i (null: i)
};

struct params_t {
  uint32_t steps;
  uint32_t tokens_per_page;
  uint64_t page_bytes;
  uint64_t budget_pages;
  uint64_t seed;
  uint32_t width;  // warp-aggregation width
};

// control words, double-buffered by step parity
struct ctrl_t {
  uint64_t next;        // first stream not admitted yet
  uint64_t k;           // streams admitted at this step
  uint64_t free_count;  // slots on the free stack
  uint64_t committed;   // pages of admitted, unfinished streams
  uint64_t live;        // pages held
  uint64_t act_n;       // active streams carried into this step
  uint64_t done_packed;  // (streams << 40) | pages of the streams that completed in phase 1
  uint64_t misses;       // page mallocs that returned NULL in phase 1
  uint64_t t_phase1;     // %globaltimer when this step's phase 1 began
  uint64_t t_phase2;     // ... and when its phase 2 began
  uint64_t pad[6];
};

struct server_t {
  ctrl_t *ctrl;           // [2]
  uint32_t *act;          // [2][slots] active slot lists
  uint32_t *done_list;    // [slots]
  uint32_t *done_off;     // [slots] first page of each finished stream in the step's flat page list
  uint32_t *free_stack;   // [slots]
  uint32_t *slot_stream;  // [slots]
  uint32_t *slot_pages;   // [slots] pages held
  uint64_t *page_table;   // [slots][max_pages]
  uint32_t slots;
  uint32_t max_pages;
};

struct out_t {
  uint64_t *checksum;        // [n] over the tokens read back at completion
  uint32_t *admit_step;      // [n]
  uint32_t *finish_step;     // [n]
  uint64_t *step_stats;      // [steps][kStats]
  unsigned long long *hist;  // [kHistBuckets] page-malloc latency, ns
};

enum { STAT_ALLOC = 0, STAT_DONE = 1, STAT_FREED = 2, STAT_LIVE = 3, STAT_COMMITTED = 4, STAT_QUEUED = 5,
       STAT_OWNED_SEGMENTS = 6, STAT_MISSES = 7, STAT_PHASE1_NS = 8, STAT_PHASE2_NS = 9, kStats = 10 };

// Segments the allocator holds (formatted or in multi-segment allocations),
// when it can say; ~0 otherwise.
template <class A>
__device__ __forceinline__ auto owned_segments(A *a, int) -> decltype(a->owned_segments()) {
  return a->owned_segments();
}
template <class A>
__device__ __forceinline__ uint64_t owned_segments(A *, long) {
  return ~0ull;
}

// Largest k <= kmax with prefix[next + k] - prefix[next] <= room.
__device__ inline uint64_t admit_count(const uint64_t *prefix, uint64_t next, uint64_t kmax, uint64_t room) {
  const uint64_t lim = prefix[next] + room;
  uint64_t lo = 0, hi = kmax;
  while (lo < hi) {
    const uint64_t mid = (lo + hi + 1) >> 1;
    if (prefix[next + mid] <= lim) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ctrl[0] for step 0: nothing admitted yet, every slot free.
__device__ inline void prologue(const server_t &sv, const trace_t &tr, const params_t &pr) {
  ctrl_t &c = sv.ctrl[0];
  const uint64_t arrived = tr.arrivals_end[1];
  const uint64_t kmax = arrived < c.free_count ? arrived : c.free_count;
  c.k = admit_count(tr.page_prefix, 0, kmax, pr.budget_pages);
  c.committed = tr.page_prefix[c.k];
}

// One stream's page for this step (phase 1).
template <class A>
__device__ inline void take_page(A *a, const server_t &sv, const trace_t &tr, const params_t &pr, const out_t &out,
                                 uint32_t s, uint32_t slot, uint32_t stream, bool fresh, uint32_t *s_hist) {
  const uint32_t par = s & 1;
  uint32_t j = 0;
  if (fresh) {
    sv.slot_stream[slot] = stream;
    out.admit_step[stream] = s;
  } else {
    j = sv.slot_pages[slot];
  }
  const uint64_t t0 = globaltimer();
  uint64_t *p = (uint64_t *)galwork::wl_malloc(a, pr.page_bytes, pr.width, 0);
  const uint64_t t1 = globaltimer();
  atomicAdd(s_hist + hist_bucket(t1 - t0), 1u);
  const uint32_t npages = tr.pages[stream];
  if (p == nullptr) {
    atomicAdd((unsigned long long *)&sv.ctrl[par].misses, 1ull);  // retried next step
  } else {
    const uint32_t len = tr.tokens[stream];
    const uint32_t id = tr.ids ? tr.ids[stream] : stream;
    const uint32_t base = j * pr.tokens_per_page;
    const uint32_t cnt = len - base < pr.tokens_per_page ? len - base : pr.tokens_per_page;
    for (uint32_t t = 0; t < cnt; ++t) p[t] = token(pr.seed, id, base + t);
    sv.page_table[(uint64_t)slot * sv.max_pages + j] = (uint64_t)p;
    ++j;
  }
  sv.slot_pages[slot] = j;
  if (j == npages) {
    // one atomic hands out the stream's index and the offset of its pages, so
    // the offsets rise with the index
    const uint64_t packed =
        atomicAdd((unsigned long long *)&sv.ctrl[par].done_packed, (1ull << 40) | (unsigned long long)npages);
    const uint64_t idx = packed >> 40;
    sv.done_list[idx] = slot;
    sv.done_off[idx] = (uint32_t)(packed & ((1ull << 40) - 1));
  } else {
    const uint64_t idx = atomicAdd((unsigned long long *)&sv.ctrl[par ^ 1].act_n, 1ull);
    sv.act[(uint64_t)(par ^ 1) * sv.slots + idx] = slot;
  }
}

template <class A>
__device__ inline void phase1(A *a, const server_t &sv, const trace_t &tr, const params_t &pr, const out_t &out,
                              uint32_t s, uint64_t rank, uint64_t nthreads, uint32_t *s_hist) {
  const ctrl_t &c = sv.ctrl[s & 1];
  const uint64_t n = c.act_n, k = c.k, free_count = c.free_count, next = c.next;
  if (rank == 0) {
    const uint64_t t = globaltimer();
    sv.ctrl[s & 1].t_phase1 = t;
    if (s > 0) out.step_stats[(uint64_t)(s - 1) * kStats + STAT_PHASE2_NS] = t - sv.ctrl[(s & 1) ^ 1].t_phase2;
  }
  for (uint64_t i = rank; i < n + k; i += nthreads) {
    if (i < n) {
      const uint32_t slot = sv.act[(uint64_t)(s & 1) * sv.slots + i];
      take_page(a, sv, tr, pr, out, s, slot, sv.slot_stream[slot], false, s_hist);
    } else {
      const uint64_t q = i - n;
      const uint32_t slot = sv.free_stack[free_count - 1 - q];
      take_page(a, sv, tr, pr, out, s, slot, (uint32_t)(next + q), true, s_hist);
    }
  }
}

// Free the pages of a slot with the whole CTA (a stream holds up to
// max_pages pages); returns to thread 0 the checksum of the tokens read back
// (when `sum`). Every thread of the CTA calls it.
template <class A>
__device__ inline uint64_t release_pages(A *a, const server_t &sv, const params_t &pr, uint32_t slot, uint32_t len,
                                         uint32_t held, bool sum, uint64_t *s_red) {
  uint64_t acc = 0;
  for (uint32_t j = threadIdx.x; j < held; j += blockDim.x) {
    uint64_t *p = (uint64_t *)sv.page_table[(uint64_t)slot * sv.max_pages + j];
    if (sum) {
      const uint32_t base = j * pr.tokens_per_page;
      const uint32_t cnt = len - base < pr.tokens_per_page ? len - base : pr.tokens_per_page;
      for (uint32_t t = 0; t < cnt; ++t) acc += p[t] * (2ull * (base + t) + 1);
    }
    galwork::wl_free(a, (void *)p, pr.width, 0);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0)
    for (uint32_t w = 1; w < (blockDim.x >> 5); ++w) acc += s_red[w];
  __syncthreads();
  return acc;
}

// Finished streams' pages as one flat list, spread over every thread: page f
// belongs to the finished stream whose first page is the last done_off <= f.
// Each thread reads back its page's tokens, adds them to the stream's
// checksum (a sum mod 2^64, so the order of the adds does not matter) and
// frees the page; the thread with a stream's first page returns its slot.
template <class A>
__device__ inline void release_flat(A *a, const server_t &sv, const trace_t &tr, const params_t &pr,
                                    const out_t &out, uint32_t s, uint64_t done, uint64_t pages, uint64_t base,
                                    uint64_t rank, uint64_t nthreads) {
  for (uint64_t f = rank; f < pages; f += nthreads) {
    uint64_t lo = 0, hi = done - 1;
    while (lo < hi) {
      const uint64_t mid = (lo + hi + 1) >> 1;
      if (sv.done_off[mid] <= f) lo = mid;
      else hi = mid - 1;
    }
    const uint32_t slot = sv.done_list[lo];
    const uint32_t stream = sv.slot_stream[slot];
    const uint32_t j = (uint32_t)(f - sv.done_off[lo]);
    const uint64_t *p = (const uint64_t *)sv.page_table[(uint64_t)slot * sv.max_pages + j];
    const uint32_t len = tr.tokens[stream];
    const uint32_t first = j * pr.tokens_per_page;
    const uint32_t cnt = len - first < pr.tokens_per_page ? len - first : pr.tokens_per_page;
    uint64_t acc = 0;
    for (uint32_t t = 0; t < cnt; ++t) acc += p[t] * (2ull * (first + t) + 1);
    atomicAdd((unsigned long long *)out.checksum + stream, (unsigned long long)acc);
    galwork::wl_free(a, (void *)p, pr.width, 0);
    if (j == 0) {
      out.finish_step[stream] = s;
      sv.free_stack[base + lo] = slot;
    }
  }
}

template <class A>
__device__ inline void phase2(A *a, const server_t &sv, const trace_t &tr, const params_t &pr, const out_t &out,
                              uint32_t s, uint64_t rank, uint64_t nthreads) {
  const uint32_t par = s & 1;
  const uint64_t t2 = rank == 0 ? globaltimer() : 0;  // phase 2 begins
  const ctrl_t &c = sv.ctrl[par];
  const uint64_t base = c.free_count - c.k;  // free-stack top after this step's pops
  const uint64_t packed = c.done_packed;
  const uint64_t done = packed >> 40, done_pages = packed & ((1ull << 40) - 1);
  if (done) release_flat(a, sv, tr, pr, out, s, done, done_pages, base, rank, nthreads);
  if (rank == 0) {
    ctrl_t &nc = sv.ctrl[par ^ 1];
    const uint64_t alloc = c.act_n + c.k - c.misses;
    nc.next = c.next + c.k;
    nc.free_count = base + done;
    nc.live = c.live + alloc - done_pages;
    const uint64_t committed = c.committed - done_pages;
    const uint64_t arrived = tr.arrivals_end[s + 1 < pr.steps ? s + 2 : pr.steps];
    uint64_t kmax = arrived > nc.next ? arrived - nc.next : 0;
    if (kmax > nc.free_count) kmax = nc.free_count;
    const uint64_t room = pr.budget_pages > committed ? pr.budget_pages - committed : 0;
    nc.k = s + 1 < pr.steps ? admit_count(tr.page_prefix, nc.next, kmax, room) : 0;
    nc.committed = committed + (tr.page_prefix[nc.next + nc.k] - tr.page_prefix[nc.next]);
    nc.done_packed = 0;
    nc.misses = 0;
    sv.ctrl[par].t_phase2 = t2;
    uint64_t *st = out.step_stats + (uint64_t)s * kStats;
    st[STAT_PHASE1_NS] = t2 - c.t_phase1;
    st[STAT_ALLOC] = alloc;
    st[STAT_DONE] = done;
    st[STAT_FREED] = done_pages;
    st[STAT_LIVE] = c.live + alloc;
    st[STAT_COMMITTED] = c.committed;
    st[STAT_QUEUED] = tr.arrivals_end[s + 1] - (c.next + c.k);
    st[STAT_OWNED_SEGMENTS] = owned_segments(a, 0);
    st[STAT_MISSES] = c.misses;
    sv.ctrl[par].act_n = 0;  // consumed by this step's phase 1
  }
}

// After the last step: free what the unfinished streams hold (one CTA per
// stream).
template <class A>
__device__ inline void drain(A *a, const server_t &sv, const trace_t &tr, const params_t &pr, uint64_t *s_red) {
  const uint32_t par = pr.steps & 1;
  const uint64_t n = sv.ctrl[par].act_n;
  for (uint64_t j = blockIdx.x; j < n; j += gridDim.x) {
    const uint32_t slot = sv.act[(uint64_t)par * sv.slots + j];
    const uint32_t stream = sv.slot_stream[slot];
    release_pages(a, sv, pr, slot, tr.tokens[stream], sv.slot_pages[slot], false, s_red);
    if (threadIdx.x == 0) sv.slot_stream[slot] = kEmpty;
  }
}

__device__ inline void flush_hist(const out_t &out, uint32_t *s_hist) {
  __syncthreads();
  for (int b = threadIdx.x; b < kHistBuckets; b += blockDim.x) {
    if (s_hist[b]) {
      atomicAdd(out.hist + b, (unsigned long long)s_hist[b]);
      s_hist[b] = 0;
    }
  }
  __syncthreads();
}

__device__ inline void clear_hist(uint32_t *s_hist) {
  for (int b = threadIdx.x; b < kHistBuckets; b += blockDim.x) s_hist[b] = 0;
  __syncthreads();
}

// ---- the persistent loop ---------------------------------------------------

template <class A>
__global__ void GALWORK_MIXED_BOUNDS serve_persistent_kernel(A *a, server_t sv, trace_t tr, params_t pr, out_t out) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  __shared__ uint32_t s_hist[kHistBuckets];
  __shared__ uint64_t s_red[32];
  clear_hist(s_hist);
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t rank = grid.thread_rank();
  if (rank == 0) prologue(sv, tr, pr);
  grid.sync();
  for (uint32_t s = 0; s < pr.steps; ++s) {
    phase1(a, sv, tr, pr, out, s, rank, nthreads, s_hist);
    grid.sync();
    phase2(a, sv, tr, pr, out, s, rank, nthreads);
    grid.sync();
  }
  drain(a, sv, tr, pr, s_red);
  flush_hist(out, s_hist);
}

// ---- the plain path: one launch per phase ------------------------------------

template <class A>
__global__ void serve_prologue_kernel(server_t sv, trace_t tr, params_t pr) {
  if (threadIdx.x == 0 && blockIdx.x == 0) prologue(sv, tr, pr);
}

template <class A>
__global__ void GALWORK_MIXED_BOUNDS serve_phase1_kernel(A *a, server_t sv, trace_t tr, params_t pr, out_t out,
                                                         uint32_t s) {
  __shared__ uint32_t s_hist[kHistBuckets];
  clear_hist(s_hist);
  const uint64_t rank = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  phase1(a, sv, tr, pr, out, s, rank, (uint64_t)gridDim.x * blockDim.x, s_hist);
  flush_hist(out, s_hist);
}

template <class A>
__global__ void GALWORK_MIXED_BOUNDS serve_phase2_kernel(A *a, server_t sv, trace_t tr, params_t pr, out_t out,
                                                         uint32_t s) {
  const uint64_t rank = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  phase2(a, sv, tr, pr, out, s, rank, (uint64_t)gridDim.x * blockDim.x);
}

template <class A>
__global__ void GALWORK_MIXED_BOUNDS serve_drain_kernel(A *a, server_t sv, trace_t tr, params_t pr) {
  __shared__ uint64_t s_red[32];
  drain(a, sv, tr, pr, s_red);
}

// ---- host side: scratch layout, initialisation, launch ----------------------

struct layout_t {
  uint64_t ctrl, act, done_list, done_off, free_stack, slot_stream, slot_pages, page_table, total;
};

inline uint64_t align256(uint64_t x) { return (x + 255) & ~255ull; }

inline layout_t layout(uint32_t slots, uint32_t max_pages) {
  layout_t l;
  uint64_t o = 0;
  l.ctrl = o;
  o = align256(o + 2 * sizeof(ctrl_t));
  l.act = o;
  o = align256(o + 2ull * slots * 4);
  l.done_list = o;
  o = align256(o + (uint64_t)slots * 4);
  l.done_off = o;
  o = align256(o + (uint64_t)slots * 4);
  l.free_stack = o;
  o = align256(o + (uint64_t)slots * 4);
  l.slot_stream = o;
  o = align256(o + (uint64_t)slots * 4);
  l.slot_pages = o;
  o = align256(o + (uint64_t)slots * 4);
  l.page_table = o;
  o = align256(o + (uint64_t)slots * max_pages * 8);
  l.total = o;
  return l;
}

inline server_t server_at(void *base, uint32_t slots, uint32_t max_pages) {
  const layout_t l = layout(slots, max_pages);
  char *b = (char *)base;
  server_t sv;
  sv.ctrl = (ctrl_t *)(b + l.ctrl);
  sv.act = (uint32_t *)(b + l.act);
  sv.done_list = (uint32_t *)(b + l.done_list);
  sv.done_off = (uint32_t *)(b + l.done_off);
  sv.free_stack = (uint32_t *)(b + l.free_stack);
  sv.slot_stream = (uint32_t *)(b + l.slot_stream);
  sv.slot_pages = (uint32_t *)(b + l.slot_pages);
  sv.page_table = (uint64_t *)(b + l.page_table);
  sv.slots = slots;
  sv.max_pages = max_pages;
  return sv;
}

// Fresh server state and cleared outputs for one run.
__global__ void init_kernel(server_t sv, out_t out, uint32_t n_streams, uint32_t steps) {
  const uint64_t rank = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nthreads = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = rank; i < sv.slots; i += nthreads) {
    sv.free_stack[i] = sv.slots - 1 - (uint32_t)i;  // pops hand out slots 0, 1, 2 ...
    sv.slot_stream[i] = kEmpty;
    sv.slot_pages[i] = 0;
  }
  for (uint64_t i = rank; i < n_streams; i += nthreads) {
    out.checksum[i] = 0;
    out.admit_step[i] = kEmpty;
    out.finish_step[i] = kEmpty;
  }
  for (uint64_t i = rank; i < (uint64_t)steps * kStats; i += nthreads) out.step_stats[i] = 0;
  for (uint64_t i = rank; i < (uint64_t)kHistBuckets; i += nthreads) out.hist[i] = 0;
  if (rank < 2 * sizeof(ctrl_t) / 8) ((uint64_t *)sv.ctrl)[rank] = 0;
}

__global__ void init_ctrl_kernel(server_t sv) { sv.ctrl[0].free_count = sv.slots; }

// mode 0: the plain path (one launch per phase per step); mode 1: one
// cooperative launch of `ctas` CTAs (all resident). Phase 2 and the drain of
// the plain path use `ctas` CTAs too.
template <class A>
cudaError_t run(A *a, const server_t &sv, const trace_t &tr, const params_t &pr, const out_t &out, uint32_t mode,
                uint32_t ctas, cudaStream_t s) {
  init_kernel<<<ctas, 256, 0, s>>>(sv, out, tr.n_streams, pr.steps);
  init_ctrl_kernel<<<1, 1, 0, s>>>(sv);
  if (mode == 1) {
    A *ap = a;
    server_t svc = sv;
    trace_t trc = tr;
    params_t prc = pr;
    out_t outc = out;
    void *args[] = {&ap, &svc, &trc, &prc, &outc};
    return cudaLaunchCooperativeKernel((const void *)serve_persistent_kernel<A>, dim3(ctas), dim3(256), args, 0, s);
  }
  serve_prologue_kernel<A><<<1, 32, 0, s>>>(sv, tr, pr);
  const unsigned items = (unsigned)((sv.slots + 255) / 256);  // a thread per slot that can be active
  for (uint32_t step = 0; step < pr.steps; ++step) {
    serve_phase1_kernel<A><<<items, 256, 0, s>>>(a, sv, tr, pr, out, step);
    serve_phase2_kernel<A><<<ctas, 256, 0, s>>>(a, sv, tr, pr, out, step);
  }
  serve_drain_kernel<A><<<ctas, 256, 0, s>>>(a, sv, tr, pr);
  return cudaGetLastError();
}

}  // namespace galserve

#endif  // GALLATIN_GB300_SERVING_CUH

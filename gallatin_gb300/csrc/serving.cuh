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
// %globaltimer); on the same threads, the pages of the streams that finished
// at step s - 1 are read back and freed, a page per thread, overlapping the
// step's mallocs. Phase 2: those streams' slots go back on the free stack,
// and thread 0 computes k_{s+1}: the longest arrival-ordered run of waiting
// streams that have arrived, fit in the free slots, and whose pages fit in
// the page budget beside the pages committed to admitted streams that have
// not finished. A stream finishing at step s gives back its pages for the
// admission of step s + 1 and its slot (once its pages are freed) for step
// s + 2. Admission therefore needs no
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
  uint64_t free_count;  // clean slots on the free stack
  uint64_t committed;   // pages of admitted streams that have not finished
  uint64_t live;        // pages held at the start of the step
  uint64_t act_n;       // active streams carried into this step
  uint64_t misses;      // page mallocs that returned NULL in phase 1
  uint64_t t_phase1;    // %globaltimer when this step's phase 1 began
  uint64_t t_phase2;    // ... and when its phase 2 began
  uint64_t pad[7];
};

// Streams that finished at step s are listed in done list s % 3: read back and
// freed during step s + 1's phase 1, their slots returned in step s + 1's
// phase 2, the list cleared in step s + 2's phase 2 for step s + 3.
struct server_t {
  ctrl_t *ctrl;             // [2]
  uint64_t *done_packed;    // [3] (streams << 40) | pages of each done list
  uint32_t *act;            // [2][slots] active slot lists
  uint32_t *done_list;      // [3][slots]
  uint32_t *done_off;       // [3][slots] first page of each finished stream in its list's flat page range
  uint32_t *free_stack;     // [slots]
  uint32_t *slot_stream;    // [slots]
  uint32_t *slot_pages;     // [slots] pages held
  uint64_t *page_table;     // [slots][max_pages]
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

constexpr uint64_t kPagesMask = (1ull << 40) - 1;

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
// the same, counted by the 32 lanes of a converged warp
template <class A>
__device__ __forceinline__ auto owned_segments_warp(A *a, uint32_t lane, int) -> decltype(a->owned_segments_warp(lane)) {
  return a->owned_segments_warp(lane);
}
template <class A>
__device__ __forceinline__ uint64_t owned_segments_warp(A *a, uint32_t, long) {
  return owned_segments(a, 0);
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

// The same with the 32 lanes of a converged warp: each round probes 32
// evenly spaced candidates, so about four rounds cover a million streams.
__device__ inline uint64_t admit_count_warp(const uint64_t *prefix, uint64_t next, uint64_t kmax, uint64_t room) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t lim = prefix[next] + room;
  uint64_t lo = 0, hi = kmax;  // the answer is in [lo, hi]
  for (int round = 0; round < 16 && lo < hi; ++round) {
    const uint64_t span = hi - lo;
    const uint64_t stride = (span + 31) / 32;
    const uint64_t x = lo + (uint64_t)(lane + 1) * stride;
    const bool ok = x <= hi && prefix[next + x] <= lim;
    const uint32_t pass = __ballot_sync(0xffffffffu, ok);
    if (pass) {
      const uint32_t l = 31 - __clz(pass);  // candidates pass as a prefix of the lanes
      lo = lo + (uint64_t)(l + 1) * stride;
      const uint64_t bound = lo + stride - 1;
      hi = bound < hi ? bound : hi;
    } else {
      hi = lo + stride - 1 < hi ? lo + stride - 1 : hi;
    }
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
    const uint32_t d = s % 3;
    const uint64_t packed =
        atomicAdd((unsigned long long *)sv.done_packed + d, (1ull << 40) | (unsigned long long)npages);
    const uint64_t idx = packed >> 40;
    sv.done_list[(uint64_t)d * sv.slots + idx] = slot;
    sv.done_off[(uint64_t)d * sv.slots + idx] = (uint32_t)(packed & kPagesMask);
    out.finish_step[stream] = s;
  } else {
    const uint64_t idx = atomicAdd((unsigned long long *)&sv.ctrl[par ^ 1].act_n, 1ull);
    sv.act[(uint64_t)(par ^ 1) * sv.slots + idx] = slot;
  }
}

// Page f of done list d (the finished streams' pages as one flat range):
// read its tokens back into the stream's checksum (a sum mod 2^64, so the
// order of the adds does not matter) and free it.
template <class A>
__device__ inline void release_page(A *a, const server_t &sv, const trace_t &tr, const params_t &pr,
                                    const out_t &out, uint32_t d, uint64_t done, uint64_t f) {
  const uint32_t *off = sv.done_off + (uint64_t)d * sv.slots;
  uint64_t lo = 0, hi = done - 1;
  while (lo < hi) {
    const uint64_t mid = (lo + hi + 1) >> 1;
    if (off[mid] <= f) lo = mid;
    else hi = mid - 1;
  }
  const uint32_t slot = sv.done_list[(uint64_t)d * sv.slots + lo];
  const uint32_t stream = sv.slot_stream[slot];
  const uint32_t j = (uint32_t)(f - off[lo]);
  const uint64_t *p = (const uint64_t *)sv.page_table[(uint64_t)slot * sv.max_pages + j];
  const uint32_t len = tr.tokens[stream];
  const uint32_t first = j * pr.tokens_per_page;
  const uint32_t cnt = len - first < pr.tokens_per_page ? len - first : pr.tokens_per_page;
  uint64_t acc = 0;
  for (uint32_t t = 0; t < cnt; ++t) acc += p[t] * (2ull * (first + t) + 1);
  atomicAdd((unsigned long long *)out.checksum + stream, (unsigned long long)acc);
  galwork::wl_free(a, (void *)p, pr.width, 0);
}

// Phase 1 of step s: a page for every active and newly admitted stream, and,
// on the same threads, the pages of the streams that finished at step s - 1.
template <class A>
__device__ inline void phase1(A *a, const server_t &sv, const trace_t &tr, const params_t &pr, const out_t &out,
                              uint32_t s, uint64_t rank, uint64_t nthreads, uint32_t *s_hist) {
  const ctrl_t &c = sv.ctrl[s & 1];
  const uint64_t n = c.act_n, k = c.k, free_count = c.free_count, next = c.next;
  const uint32_t dprev = (s + 2) % 3;
  const uint64_t packed = s > 0 ? sv.done_packed[dprev] : 0;
  const uint64_t done = packed >> 40, pages = packed & kPagesMask;
  if (rank == 0) {
    const uint64_t t = globaltimer();
    sv.ctrl[s & 1].t_phase1 = t;
    if (s > 0) out.step_stats[(uint64_t)(s - 1) * kStats + STAT_PHASE2_NS] = t - sv.ctrl[(s & 1) ^ 1].t_phase2;
  }
  for (uint64_t i = rank; i < n + k + pages; i += nthreads) {
    if (i < n) {
      const uint32_t slot = sv.act[(uint64_t)(s & 1) * sv.slots + i];
      take_page(a, sv, tr, pr, out, s, slot, sv.slot_stream[slot], false, s_hist);
    } else if (i < n + k) {
      const uint64_t q = i - n;
      const uint32_t slot = sv.free_stack[free_count - 1 - q];
      take_page(a, sv, tr, pr, out, s, slot, (uint32_t)(next + q), true, s_hist);
    } else {
      release_page(a, sv, tr, pr, out, dprev, done, i - n - k);
    }
  }
}

// Phase 2 of step s: the slots of the streams that finished at step s - 1
// (their pages freed in this step's phase 1) go back on the free stack;
// thread 0 admits for step s + 1.
template <class A>
__device__ inline void phase2(A *a, const server_t &sv, const trace_t &tr, const params_t &pr, const out_t &out,
                              uint32_t s, uint64_t rank, uint64_t nthreads) {
  const uint32_t par = s & 1;
  const uint64_t t2 = rank < 32 ? globaltimer() : 0;  // phase 2 begins
  const ctrl_t &c = sv.ctrl[par];
  const uint64_t base = c.free_count - c.k;  // free-stack top after this step's pops
  const uint32_t dprev = (s + 2) % 3;
  const uint64_t prev = s > 0 ? sv.done_packed[dprev] : 0;
  const uint64_t prev_done = prev >> 40, prev_pages = prev & kPagesMask;
  for (uint64_t j = rank; j < prev_done; j += nthreads)
    sv.free_stack[base + j] = sv.done_list[(uint64_t)dprev * sv.slots + j];
  if (rank < 32) {  // warp 0 of CTA 0: admission for step s + 1 and the step's stats
    __syncwarp();
    const uint32_t lane = (uint32_t)rank;
    const uint64_t cur = sv.done_packed[s % 3];  // finished at s: pages freed at s + 1
    const uint64_t done = cur >> 40, done_pages = cur & kPagesMask;
    const uint64_t alloc = c.act_n + c.k - c.misses;
    const uint64_t next = c.next + c.k;
    const uint64_t free_count = base + prev_done;
    const uint64_t committed = c.committed - done_pages;
    const uint64_t arrived = tr.arrivals_end[s + 1 < pr.steps ? s + 2 : pr.steps];
    uint64_t kmax = arrived > next ? arrived - next : 0;
    if (kmax > free_count) kmax = free_count;
    const uint64_t room = pr.budget_pages > committed ? pr.budget_pages - committed : 0;
    const uint64_t k = s + 1 < pr.steps ? admit_count_warp(tr.page_prefix, next, kmax, room) : 0;
    const uint64_t owned = owned_segments_warp(a, lane, 0);
    if (lane == 0) {
      ctrl_t &nc = sv.ctrl[par ^ 1];
      nc.next = next;
      nc.free_count = free_count;
      nc.live = c.live + alloc - prev_pages;
      nc.k = k;
      nc.committed = committed + (tr.page_prefix[next + k] - tr.page_prefix[next]);
      nc.misses = 0;
      sv.done_packed[(s + 1) % 3] = 0;  // step s - 2's list, done with in step s - 1; refilled at step s + 1
      sv.ctrl[par].t_phase2 = t2;
      uint64_t *st = out.step_stats + (uint64_t)s * kStats;
      st[STAT_PHASE1_NS] = t2 - c.t_phase1;
      st[STAT_ALLOC] = alloc;
      st[STAT_DONE] = done;
      st[STAT_FREED] = prev_pages;
      st[STAT_LIVE] = nc.live;
      st[STAT_COMMITTED] = c.committed;
      st[STAT_QUEUED] = tr.arrivals_end[s + 1] - (c.next + c.k);
      st[STAT_OWNED_SEGMENTS] = owned;
      st[STAT_MISSES] = c.misses;
      sv.ctrl[par].act_n = 0;  // consumed by this step's phase 1
    }
  }
}

// Free the pages of a slot with the whole CTA (every thread of the CTA calls it).
template <class A>
__device__ inline void release_slot_cta(A *a, const server_t &sv, const params_t &pr, uint32_t slot, uint32_t held) {
  for (uint32_t j = threadIdx.x; j < held; j += blockDim.x)
    galwork::wl_free(a, (void *)sv.page_table[(uint64_t)slot * sv.max_pages + j], pr.width, 0);
}

// After the last step: read back and free the streams that finished at the
// last step, and free what the unfinished streams hold.
template <class A>
__device__ inline void drain(A *a, const server_t &sv, const trace_t &tr, const params_t &pr, const out_t &out,
                             uint64_t rank, uint64_t nthreads) {
  const uint32_t dlast = (pr.steps - 1) % 3;
  const uint64_t packed = sv.done_packed[dlast];
  const uint64_t done = packed >> 40, pages = packed & kPagesMask;
  for (uint64_t f = rank; f < pages; f += nthreads) release_page(a, sv, tr, pr, out, dlast, done, f);
  const uint32_t par = pr.steps & 1;
  const uint64_t n = sv.ctrl[par].act_n;
  for (uint64_t j = blockIdx.x; j < n; j += gridDim.x) {
    const uint32_t slot = sv.act[(uint64_t)par * sv.slots + j];
    release_slot_cta(a, sv, pr, slot, sv.slot_pages[slot]);
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
  drain(a, sv, tr, pr, out, rank, nthreads);
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
__global__ void GALWORK_MIXED_BOUNDS serve_drain_kernel(A *a, server_t sv, trace_t tr, params_t pr, out_t out) {
  const uint64_t rank = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  drain(a, sv, tr, pr, out, rank, (uint64_t)gridDim.x * blockDim.x);
}

// ---- host side: scratch layout, initialisation, launch ----------------------

struct layout_t {
  uint64_t ctrl, done_packed, act, done_list, done_off, free_stack, slot_stream, slot_pages, page_table, total;
};

inline uint64_t align256(uint64_t x) { return (x + 255) & ~255ull; }

inline layout_t layout(uint32_t slots, uint32_t max_pages) {
  layout_t l;
  uint64_t o = 0;
  l.ctrl = o;
  o = align256(o + 2 * sizeof(ctrl_t));
  l.done_packed = o;
  o = align256(o + 3 * sizeof(uint64_t));
  l.act = o;
  o = align256(o + 2ull * slots * 4);
  l.done_list = o;
  o = align256(o + 3ull * slots * 4);
  l.done_off = o;
  o = align256(o + 3ull * slots * 4);
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
  sv.done_packed = (uint64_t *)(b + l.done_packed);
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
  if (rank < 3) sv.done_packed[rank] = 0;
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
  serve_drain_kernel<A><<<ctas, 256, 0, s>>>(a, sv, tr, pr, out);
  return cudaGetLastError();
}

}  // namespace galserve

#endif  // GALLATIN_GB300_SERVING_CUH

/*
 * gallatin_gb300 C ABI.
 *
 * Host entry points of the GB300 Gallatin allocator, behind plain C types:
 * handles, pointers, sizes and a cudaStream_t passed as void*. No torch or
 * C++ types cross this boundary. The device-side malloc/free that user
 * kernels call are header-only (include/gallatin/allocators/gallatin.cuh);
 * this library creates, inspects and destroys the state they operate on,
 * and runs batch and benchmark kernels over it.
 *
 * Each entry names the reference interface it replaces (paths inside the
 * saltsystemslab/gallatin tree). Calls on one handle are not thread-safe;
 * different handles are independent. Every function returns GAL_OK or a
 * GAL_ERR_* code; nothing here calls exit() or traps.
 */
#ifndef GALLATIN_GB300_H
#define GALLATIN_GB300_H

#include <stdint.h>

#include "gallatin_gb300/state.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GAL_OK 0
#define GAL_ERR_INVALID 1   /* bad argument or unsupported geometry */
#define GAL_ERR_CUDA 2      /* a CUDA runtime call failed */
#define GAL_ERR_NOMEM 3     /* device or host allocation failed */

typedef struct gal_allocator gal_allocator; /* opaque host handle */
typedef struct gal_veb gal_veb;             /* opaque standalone vEB tree */

typedef struct gal_geometry_t {
  uint64_t segment_bytes;
  uint64_t min_size;
  uint64_t max_size;
  uint64_t num_segments;
  uint64_t arena_bytes;
  uint32_t num_trees;
  uint32_t blocks_per_segment;
  uint32_t num_sms;
  uint32_t total_slots;
  uint32_t slot_count[GAL_MAX_TREES]; /* per slot class */
  uint32_t num_classes;               /* slot classes: num_trees - 1 single-slice
                                         trees, then one per run length 1, 2, 4 ...
                                         of the largest tree */
  uint32_t flags;      /* GAL_FLAG_* the allocator was created with */
  uint64_t arena_base; /* device address of the arena (with GAL_FLAG_HOST_ARENA
                          also its host address: the mapping is the identity) */
} gal_geometry_t;

typedef struct gal_stats_t {
  uint64_t num_segments;
  uint64_t free_segments;                    /* set leaf bits of the segment tree */
  uint64_t tree_segments[GAL_MAX_TREES];     /* segments formatted for tree t */
  uint64_t tree_blocks_out[GAL_MAX_TREES];   /* blocks of tree t not in a segment pool */
  uint64_t tree_live_slices[GAL_MAX_TREES];  /* live count summed over those blocks */
  uint64_t segment_allocations;              /* live multi-segment allocations */
  uint64_t segments_in_allocations;          /* segments they span */
  uint64_t counters[GAL_NUM_COUNTERS];
} gal_stats_t;

/* --- allocator lifetime (reference gallatin.cuh:324-421, :643-668) --- */

/* Build an allocator over max_bytes / segment_bytes segments. segment_bytes,
 * min_size and max_size must be powers of two with
 * segment_bytes >= max_size * 4096 (reference static_assert gallatin.cuh:300)
 * and max_size >= 32 * min_size (multi-slice runs fit one bitmap word).
 * min_slots: floor on pinned blocks per slot class (0 = default 4); the
 * count per class is otherwise one per SM, capped so a class's pinned blocks
 * take at most a quarter of the arena divided by the number of trees.
 * Replaces Gallatin<seg,min,max>::generate_on_device. */
int gal_create(uint64_t max_bytes, uint64_t seed, uint64_t segment_bytes, uint64_t min_size, uint64_t max_size,
               uint32_t min_slots, gal_allocator **out);

/* gal_create with flags, a bit set of GAL_FLAG_HOST_ARENA, GAL_FLAG_CALLOC and
 * GAL_FLAG_DROP_FREED (state.h):
 *   GAL_FLAG_DROP_FREED  a free of one slice of 128 B to 4 KiB (HBM arena,
 *                        not calloc) drops that slice's lines from L2 without
 *                        writing them back to HBM; the bytes are indeterminate
 *                        afterwards, as freed bytes are. For work that shares
 *                        HBM bandwidth: on the mixed workload it cut HBM writes
 *                        11 times and cost 11 % of the step. No counterpart
 *                        in the reference, whose free leaves the lines.
 *   GAL_FLAG_HOST_ARENA  the arena is pinned, mapped host memory; the vEB
 *                        trees, block words and bitmaps stay in HBM.
 *                        Replaces Gallatin<...>::generate_on_device_host
 *                        (reference gallatin.cuh:423-526, arena from
 *                        memory_table.cuh:521-540).
 *   GAL_FLAG_CALLOC      malloc returns zeroed bytes: the arena is zeroed
 *                        here and every free zeroes what it returns before
 *                        the bytes can be handed out again (reference
 *                        running_calloc, gallatin.cuh:324-325,1306-1369).
 * gal_create(...) is gal_create_ex(..., 0, out). */
int gal_create_ex(uint64_t max_bytes, uint64_t seed, uint64_t segment_bytes, uint64_t min_size, uint64_t max_size,
                  uint32_t min_slots, uint32_t flags, gal_allocator **out);

/* Free everything, arena included (reference free_on_device, gallatin.cuh:643). */
int gal_destroy(gal_allocator *h);

/* Device pointer to the allocator state: the value generate_on_device
 * returns and user kernels receive (reference gallatin.cuh:419). */
void *gal_device_state(gal_allocator *h);

/* Handle owning a device state pointer, or NULL. Lets the header-only
 * Gallatin<...> template map its device pointer back (reference
 * free_on_device/print_info take the device pointer, gallatin.cuh:643,1855). */
gal_allocator *gal_from_device_state(const void *device_state);

int gal_geometry(gal_allocator *h, gal_geometry_t *out);

/* --- stats (reference print_info gallatin.cuh:1855-1897,
 *     report_fill veb.cuh:1052, print_global_stats global_allocator.cuh:86) --- */
int gal_stats(gal_allocator *h, gal_stats_t *out);
int gal_print_info(gal_allocator *h);
int gal_reset_counters(gal_allocator *h);

/* Copy one metadata array to host memory for invariant checks.
 * which: see GAL_DUMP_*; tree selects the sub tree for GAL_DUMP_SUB_TREE
 * and layer the vEB layer. gal_dump_bytes gives the size to provide. */
#define GAL_DUMP_CHUNK_IDS 0
#define GAL_DUMP_SEG_AVAIL 1
#define GAL_DUMP_SEG_BLOCK_BITS 2
#define GAL_DUMP_BLOCK_META 3
#define GAL_DUMP_BLOCK_BITS 4
/* 5 is unused */
#define GAL_DUMP_SLOTS 6
#define GAL_DUMP_COUNTERS 7
#define GAL_DUMP_SEGMENT_TREE 8
#define GAL_DUMP_SUB_TREE 9
#define GAL_DUMP_LOCKS 10
#define GAL_DUMP_ADOPT_TREE 11
#define GAL_DUMP_ROOMY_TREE 12
int64_t gal_dump_bytes(gal_allocator *h, int which, int tree, int layer);
int gal_dump(gal_allocator *h, int which, int tree, int layer, void *host_dst, uint64_t bytes);
/* layers of a vEB tree of this allocator: which is GAL_DUMP_SEGMENT_TREE,
 * GAL_DUMP_SUB_TREE (tree selects the size class), GAL_DUMP_ADOPT_TREE or
 * GAL_DUMP_ROOMY_TREE (tree selects the slot class) */
int gal_veb_layer_count(gal_allocator *h, int which, int tree);

/* End-state check: after every allocation is freed and gal_flush_pinned
 * has run (no kernel running), compare every tree and table with the state
 * gal_create left and count the differences. The reference has no such
 * check; its tests count live slices per block (tests/src/
 * gallatin_host_test.cu:87-95, check_overlaps_kernel). restored is 1 when
 * every count is zero. */
typedef struct gal_restore_report_t {
  uint64_t segment_tree_words; /* segment tree words that differ from a full tree */
  uint64_t sub_tree_words;     /* non-zero words of the per-size sub trees */
  uint64_t adopt_tree_words;   /* non-zero words of the adoptable and roomy trees */
  uint64_t tagged_segments;    /* memory-table entries not marked free */
  uint64_t open_segments;      /* segments whose free-block count is not at the gate */
  uint64_t blocks_out;         /* blocks not in their segment's pool */
  uint64_t live_blocks;        /* blocks whose live count is not zero */
  uint64_t taken_slices;       /* slices whose bitmap bit is not back to free */
  uint64_t pinned_slots;       /* pinned-block slots not empty */
  uint64_t corrupt;            /* GAL_CTR_CORRUPT */
  uint64_t bad_frees;          /* GAL_CTR_BAD_FREE */
  uint32_t locks;              /* the lock word */
  uint32_t restored;
} gal_restore_report_t;
int gal_check_restored(gal_allocator *h, gal_restore_report_t *out);

/* Bound on the segment-tier lock wait: a segment-tier malloc (a request
 * larger than one segment) that cannot take the lock in lock_spins tries
 * (with a backoff growing to ~1 us per try) returns NULL and counts
 * GAL_CTR_TIMEOUT. Default GAL_DEFAULT_LOCK_SPINS, about a second; no kernel
 * may run during the call. The reference waits on this lock without bound
 * (gallatin.cuh:796). */
int gal_set_wait_limit(gal_allocator *h, uint32_t lock_spins);

/* Overwrite the lock word (bit t: tree t's segment-attach lock, bit 31: the
 * segment-tier lock) while no kernel runs. A bit set here is held by no
 * thread, so every wait on it runs to its bound: this is how the tests show
 * that the waits end, without a GPU fault or hang. Clear it again (0)
 * before normal use. No counterpart in the reference. */
int gal_set_locks(gal_allocator *h, uint32_t locks);

/* --- batch entry points (device buffers, one thread per request) ---
 * These are the host-callable form of Gallatin::malloc / free
 * (gallatin.cuh:1186,1378), as the reference tests drive them from
 * kernels (tests/src/gallatin_test.cu:58-112). */
int gal_malloc_batch(gal_allocator *h, const uint64_t *d_sizes, uint64_t n, uint64_t *d_ptrs, void *stream);
int gal_free_batch(gal_allocator *h, const uint64_t *d_ptrs, uint64_t n, void *stream);

/* Size classing as the device computes it, one entry per request size:
 * tier 0 = slices (tree = size class, count = slices per request), 1 = a
 * whole block (tree = block tree, count 1), 2 = contiguous segments
 * (count = segments); allocated = the bytes the request occupies. Replaces
 * the reference's device get_tree_id_from_size / malloc dispatch /
 * get_allocated_size (gallatin.cuh:1141-1183, 1196-1260), which have no host
 * entry point there. d_sizes and d_out are device buffers of n entries. */
typedef struct gal_size_info_t {
  uint32_t tier;
  uint32_t tree;
  uint64_t count;
  uint64_t allocated;
} gal_size_info_t;
int gal_size_classes(gal_allocator *h, const uint64_t *d_sizes, uint64_t n, gal_size_info_t *d_out, void *stream);

/* L2 atomic throughput probe (the denominator of the allocator's atomic
 * roofline; no counterpart in the reference). ctas_per_sm CTAs of 256 threads
 * per SM; lane 0 of each warp issues `iters` rounds of 8 independent 64-bit
 * atomic adds, each to its own 128-byte line of d_words (lines * 128 bytes,
 * lines a power of two, at least the number of warps): mode 0 atom (returns
 * the old value, as the allocator's reservations do), mode 1 red (no return,
 * as its bitmap returns do). *ops_out = atomics the launch issues; time it on
 * `stream` with events. d_sink: one device u64 the kernel may write. */
int gal_probe_l2_atomics(uint64_t *d_words, uint64_t lines, uint32_t iters, uint32_t mode, uint32_t ctas_per_sm,
                         unsigned long long *d_sink, uint64_t *ops_out, void *stream);

/* Detach every pinned block (no malloc/free may run concurrently). Empty
 * blocks and segments return to their pools, so after all allocations are
 * freed the trees equal their initial state. No reference counterpart: the
 * reference keeps its boot-time pinned blocks forever (gallatin.cuh:171). */
int gal_flush_pinned(gal_allocator *h, void *stream);

/* --- workloads over the device API (benchmarks and e2e) ---
 * stats (device, 8 x u64): [0] slice/block misses (nullptr), [1] verify
 * failures, [2] segment-tier successes, [3] segment-tier misses.
 * Replaces the reference test kernels gallatin_test.cu:58-112 and
 * gallatin_churn.cu:36-95 as benchmark drivers. */
int gal_run_pairs(gal_allocator *h, uint64_t n_threads, uint64_t size, uint32_t block_dim,
                  unsigned long long *d_stats, void *stream);
int gal_run_mixed(gal_allocator *h, uint64_t n_threads, uint32_t rounds, uint64_t seed, uint32_t seg_every,
                  uint64_t seg_lo, uint64_t seg_hi, const uint8_t *d_classes, uint32_t block_dim,
                  unsigned long long *d_stats, void *stream);
/* Same workload end to end from host buffers: copies the class trace
 * (rounds * n_threads bytes, round-major) to the device, runs, and copies
 * the 8 stats words back, all on `stream`, then synchronises it. */
int gal_run_mixed_host(gal_allocator *h, uint64_t n_threads, uint32_t rounds, uint64_t seed, uint32_t seg_every,
                       uint64_t seg_lo, uint64_t seg_hi, const uint8_t *h_classes, uint32_t block_dim,
                       uint64_t *h_stats, void *stream);

/* Same as gal_run_mixed_host, but the call allocates no device memory: no
 * cudaMalloc, no cudaFree, no allocating library routine. It is for callers
 * that may not allocate at run time, such as a serving loop that cannot take
 * the device-wide synchronisation a cudaMalloc implies, or a process whose
 * device memory was divided up in advance. Its scratch (the trace copy and
 * the stats words) is a fixed array of GAL_NOALLOC_TRACE_MAX_BYTES + 256
 * bytes compiled into the library, which every GPU that loads the library
 * holds until the process exits; traces larger than
 * GAL_NOALLOC_TRACE_MAX_BYTES (n_threads * rounds) are rejected with
 * GAL_ERR_INVALID. Each call looks up the array's device address
 * (cudaGetSymbolAddress). Under CUDA's default lazy module loading the first
 * call on a device also loads the module holding the array, and that is when
 * the driver takes its memory: make that first call before the device's
 * memory is divided up and before any stream capture, or set
 * CUDA_MODULE_LOADING=EAGER. All calls share the one array: calls whose GPU
 * work overlaps (other streams, other host threads) race on it. No
 * counterpart in the reference, which allocates its buffers with cudaMalloc. */
#define GAL_NOALLOC_TRACE_MAX_BYTES (2ull << 20)
int gal_run_mixed_host_noalloc(gal_allocator *h, uint64_t n_threads, uint32_t rounds, uint64_t seed,
                               uint32_t seg_every, uint64_t seg_lo, uint64_t seg_hi, const uint8_t *h_classes,
                               uint32_t block_dim, uint64_t *h_stats, void *stream);

/* --- benchmark driver of the per-thread workloads (no reference
 *     counterpart: the reference's tests time one launch with a host clock
 *     around cudaDeviceSynchronize, timer.cuh:44-78) ---
 * `warmup` untimed launches, then `steps` timed ones: before each, a write
 * of flush_bytes (larger than L2, so no step starts with a warm L2), then
 * the launch between two CUDA events on `stream`; step_ms[i] is its device
 * time. With h_classes (a pinned host class trace, mixed workload only) the
 * same steps then run end to end through gal_run_mixed_host (trace copied
 * in, stats copied out, stream synchronised) with a host clock around each:
 * e2e_step_ms[i]. stats / e2e_stats: the workload's stats words summed over
 * the timed steps ([0] NULLs, [1] verify failures, [2]/[3] segment-tier
 * successes / NULLs). */
#define GAL_BENCH_PAIRS 0 /* gal_run_pairs(n_threads, size, block_dim) */
#define GAL_BENCH_MIXED 1 /* gal_run_mixed(n_threads, rounds, seed, seg_*, d_classes, block_dim) */
typedef struct gal_bench_args_t {
  uint32_t workload;
  uint32_t block_dim;
  uint64_t n_threads;
  uint64_t size;      /* pairs: bytes per malloc */
  uint32_t rounds;    /* mixed */
  uint32_t seg_every; /* mixed: segment-tier request every seg_every-th CTA (0 = none) */
  uint64_t seed;
  uint64_t seg_lo, seg_hi;
  const uint8_t *d_classes; /* mixed: device class trace, or NULL (generated on the device) */
  const uint8_t *h_classes; /* mixed: pinned host class trace for the end-to-end leg, or NULL */
  uint32_t warmup, steps;
  uint64_t flush_bytes;
  void *stream;
} gal_bench_args_t;
typedef struct gal_bench_result_t {
  float *step_ms;     /* caller buffer of `steps` floats */
  float *e2e_step_ms; /* caller buffer of `steps` floats, or NULL without the end-to-end leg */
  uint64_t stats[8];
  uint64_t e2e_stats[8];
} gal_bench_result_t;
int gal_bench(gal_allocator *h, const gal_bench_args_t *args, gal_bench_result_t *out);

/* --- device-first allocation with a host-arena fallback ---
 * The reference pairs a device allocator with one over pinned host memory
 * and offers global_malloc_fused / global_free_fused: malloc from the device
 * arena, and from the host arena when that returns NULL; free to whichever
 * arena owns the pointer (global_allocator.cuh:128-216). This runs that
 * pattern in the fill/drain shape of tests/src/global_exceed_test.cu:38-110.
 * Fill (phase_mask bit 0): thread i mallocs 16 << class_i bytes (class_i =
 * d_classes[i], or x mod 9 of xorshift64 seeded by splitmix64(seed + i) when
 * d_classes is NULL), keeps the pointer in d_table[i] (n u64) and writes i
 * to its first and ~i to its last u64. Drain (bit 1): thread i checks both
 * words, frees d_table[i] and sets it to 0. host may be NULL (device arena
 * only) and is normally a GAL_FLAG_HOST_ARENA allocator. stats: [0] NULLs,
 * [1] verify failures, [4] allocations the host arena served. */
int gal_run_fused(gal_allocator *dev, gal_allocator *host, uint64_t n, uint64_t seed, const uint8_t *d_classes,
                  uint64_t *d_table, uint32_t phase_mask, unsigned long long *d_stats, void *stream);
/* Both phases end to end from host memory: the class trace (n bytes) is
 * copied in, the 8 stats words copied out, all on `stream`, then the stream
 * is synchronised. The pointer table is scratch owned by `dev`. */
int gal_run_fused_host(gal_allocator *dev, gal_allocator *host, uint64_t n, uint64_t seed, const uint8_t *h_classes,
                       uint64_t *h_stats, void *stream);

/* Zeroed-memory check for GAL_FLAG_CALLOC allocators (the property the
 * reference's running_calloc mode is for, gallatin.cuh:1306-1369): each of
 * n_threads threads, for `rounds` rounds, mallocs 16 << (x mod 12) bytes
 * (single slices and multi-slice runs), checks that every byte reads zero,
 * fills it with a non-zero pattern and frees it; warp 0 of every
 * big_every-th CTA (256 threads) also takes one allocation of a size uniform
 * in [big_lo, big_hi] per round through the same check (0 = none). stats:
 * [0] NULLs, [1] allocations holding a non-zero byte. */
int gal_run_zeroed(gal_allocator *h, uint64_t n_threads, uint32_t rounds, uint64_t seed, uint32_t big_every,
                   uint64_t big_lo, uint64_t big_hi, unsigned long long *d_stats, void *stream);

/* --- batched request streams (no reference counterpart: the reference only
 *     serves per-thread calls from user kernels) ---
 * A request is a u64: slot << 32 | size; size > 0 mallocs into
 * table[slot], size 0 frees table[slot]. Batch b is requests
 * [offsets[b], offsets[b+1]); offsets that decrease, a width or a mode out
 * of range give GAL_ERR_INVALID before anything is allocated or launched.
 * width (8, 16, 32) limits warp aggregation to tiles of that many lanes.
 * mode 0: one launch per batch (the plain per-thread call path); mode 1: one
 * cooperative persistent launch that serves every batch with a grid barrier
 * between batches; mode 2: as mode 1, but each batch is first
 * counting-sorted on the device by power-of-two size class (frees first), so
 * a warp's lanes share a class; the sort uses scratch the handle owns, sized
 * for the largest batch. A batch of modes 1 and 2 holds at most 2^31-1
 * requests. ctas_per_sm: CTAs of 256 threads per SM for modes 1 and 2
 * (kernel geometry; 0 = as many as fit, more is refused). stats as for the
 * workloads ([0] = mallocs that returned NULL). */
int gal_run_batches(gal_allocator *h, const uint64_t *d_reqs, const uint64_t *d_offsets, const uint64_t *h_offsets,
                    uint32_t n_batches, uint64_t *d_table, uint32_t width, uint32_t mode, uint32_t ctas_per_sm,
                    unsigned long long *d_stats, void *stream);
/* Capture the same launches once into an instantiated CUDA graph; replay it
 * with gal_graph_launch and release it with gal_graph_destroy. */
int gal_capture_batches(gal_allocator *h, const uint64_t *d_reqs, const uint64_t *d_offsets, const uint64_t *h_offsets,
                        uint32_t n_batches, uint64_t *d_table, uint32_t width, uint32_t mode, uint32_t ctas_per_sm,
                        unsigned long long *d_stats, void **graph_out);
int gal_graph_launch(void *graph_exec, void *stream);
int gal_graph_destroy(void *graph_exec);
/* End to end from host buffers: copies the requests and offsets to scratch
 * the handle owns (grown on demand), runs, copies the 8 stats words back and
 * synchronises `stream`. table_slots: size of the live-set table; every
 * request's slot must be below it (not checked: that would be a host pass
 * over every request inside the call). */
int gal_run_batches_host(gal_allocator *h, const uint64_t *h_reqs, const uint64_t *h_offsets, uint32_t n_batches,
                         uint64_t table_slots, uint32_t width, uint32_t mode, uint32_t ctas_per_sm,
                         uint64_t *h_stats, void *stream);

/* --- serving loop (no reference counterpart: the reference only serves
 *     per-thread calls from user kernels) ---
 * Streams arrive over simulated steps; a stream of L tokens takes one page
 * of page_bytes per step until it holds ceil(L / tokens_per_page) pages,
 * writing its tokens (u64 each) into each page, then reads them back into a
 * checksum (sum of token * (2 * position + 1), mod 2^64) and frees its pages.
 * Admission is first-come first-served on the device: at step s the longest
 * run of waiting streams is admitted that has arrived (arrivals_end[s + 1]),
 * fits the free slots (max_slots), and keeps the pages committed to admitted,
 * unfinished streams within budget_pages. A stream finishing at step s gives
 * back its pages for the admission of step s + 1; its pages are read back and
 * freed during step s + 1 (overlapping that step's mallocs) and its slot
 * counts as free for the admission of step s + 2. After the last step every
 * page still held is freed, so the allocator ends as it started.
 * mode 0: the plain path, one launch per phase per step (phase 1: a thread
 * per stream takes its page, and finished streams' pages are freed; phase 2:
 * slots return and admission); mode 1: every step in one cooperative
 * persistent launch. */
typedef struct gal_serve_trace_t {
  uint32_t n_streams;
  uint32_t pad_;
  const uint32_t *arrivals_end; /* device [steps + 1]: [s + 1] = arrived at steps <= s */
  const uint32_t *tokens;       /* device [n]: L per stream, arrival order */
  const uint32_t *pages;        /* device [n]: ceil(L / tokens_per_page) <= max_pages */
  const uint64_t *page_prefix;  /* device [n + 1]: pages of the streams before i */
  const uint32_t *ids;          /* device [n] or NULL: the id stream i's tokens are
                                   derived from (NULL: i), so one stream can be
                                   replayed alone with the tokens it has in a mix */
} gal_serve_trace_t;

typedef struct gal_serve_params_t {
  uint32_t steps;
  uint32_t tokens_per_page;
  uint64_t page_bytes;
  uint64_t budget_pages; /* admission cap, e.g. 0.8 * arena / page_bytes */
  uint64_t seed;         /* token values */
  uint32_t max_slots;    /* streams served at once */
  uint32_t max_pages;    /* page-table width per stream */
  uint32_t width;        /* warp-aggregation width 8, 16 or 32 */
  uint32_t mode;
  uint32_t ctas_per_sm;  /* 0 = as many as fit */
  uint32_t pad_;
} gal_serve_params_t;

#define GAL_SERVE_HIST_BUCKETS 864 /* ns < 32 exact, then 32 buckets per octave */
#define GAL_SERVE_STATS 10         /* per step: allocated, finished, freed, live,
                                      committed, queued, owned segments, NULLs,
                                      phase-1 ns, phase-2 ns (%globaltimer, from
                                      the start of one phase to the next) */
typedef struct gal_serve_out_t { /* device arrays, cleared by the call */
  uint64_t *checksum;     /* [n], 0 for streams that did not finish */
  uint32_t *admit_step;   /* [n], 0xFFFFFFFF = not admitted */
  uint32_t *finish_step;  /* [n], 0xFFFFFFFF = not finished */
  uint64_t *step_stats;   /* [steps][GAL_SERVE_STATS] */
  uint64_t *latency_hist; /* [GAL_SERVE_HIST_BUCKETS] page-malloc latency */
} gal_serve_out_t;

/* The server's slot and page tables are scratch the handle owns (grown on
 * demand: max_slots * max_pages * 8 bytes and a few arrays of max_slots). */
int gal_run_serving(gal_allocator *h, const gal_serve_trace_t *trace, const gal_serve_params_t *params,
                    const gal_serve_out_t *out, void *stream);

/* The same loop with every page malloc device-first: from `dev`, and from
 * `host` (normally a GAL_FLAG_HOST_ARENA allocator of the same segment size)
 * when that returns NULL; each free goes to the arena that owns the page (the
 * reference's global_malloc_fused / global_free_fused,
 * global_allocator.cuh:186-216). The page budget may then exceed the device
 * arena: pages past it spill to host memory. step_stats owned segments count
 * both arenas. Scratch is owned by `dev`. */
int gal_run_serving_fused(gal_allocator *dev, gal_allocator *host, const gal_serve_trace_t *trace,
                          const gal_serve_params_t *params, const gal_serve_out_t *out, void *stream);

/* --- allocator-backed data structures (reference data_structs/
 *     chaining_table.cuh:57-327 and single_vector.cuh:50-200) ---
 * A chained hash table of u64 keys and values: buckets hold chains of 120 B
 * nodes (7 keys, 7 values, next) taken from this allocator with malloc when a
 * chain is full; the bucket is MurmurHash64A(key, seed) mod nbuckets. The
 * device template is galds::chaining_table in gallatin_gb300/structures.cuh;
 * these calls run it over a batch of keys, one thread per key (or per bucket
 * for COMPACT and CLEAR). Keys come from d_keys, or when d_keys is NULL are
 * splitmix64(key_seed + i); the value of a key is splitmix64(key). Key i is in
 * the "half" when splitmix64(key_seed ^ i * 0x9E3779B97F4A7C15) is odd.
 * stats (device, 8 x u64): [0] inserts that got no node (allocator NULL),
 * [1] keys found where absent or absent where expected, [2] wrong values,
 * [3] nodes freed (COMPACT, CLEAR), [4] vector pushes. Erase is an addition:
 * the reference table has none. */
typedef struct gal_table gal_table;
#define GAL_TABLE_INSERT 0
#define GAL_TABLE_ERASE_HALF 1
#define GAL_TABLE_REINSERT_HALF 2
#define GAL_TABLE_QUERY 3            /* every key must be present */
#define GAL_TABLE_COMPACT 4          /* unlink and free nodes left with no key */
#define GAL_TABLE_CLEAR 5            /* free every node */
#define GAL_TABLE_QUERY_AFTER_ERASE 6 /* present unless in the half */
int gal_table_create(gal_allocator *h, uint64_t nbuckets, uint64_t seed, gal_table **out);
int gal_table_op(gal_table *t, uint32_t op, const uint64_t *d_keys, uint64_t n, uint64_t key_seed,
                 unsigned long long *d_stats, void *stream);
/* longest chain and total nodes (reference print_chain_stats, chaining_table.cuh:300-325) */
int gal_table_chain_stats(gal_table *t, uint64_t *max_len, uint64_t *total_nodes);
/* frees the bucket directory; CLEAR first, or the nodes stay allocated */
int gal_table_destroy(gal_table *t);
/* n per-thread vectors of u32 (galds::svector): vector v starts with a
 * backing of `start` items (rounded up to a power of two) and pushes
 * d_lengths[v] items (v * 2654435761 + i) mod 2^32, doubling its backing
 * (malloc, copy, free) when full; then checks every item and frees the
 * backing. stats: [0] mallocs that returned NULL, [2] wrong items, [4] pushes. */
int gal_run_vectors(gal_allocator *h, const uint32_t *d_lengths, uint64_t n, uint32_t start,
                    unsigned long long *d_stats, void *stream);

/* --- standalone vEB tree (reference veb_tree, veb.cuh:528-1228) --- */

typedef struct gal_veb_op {
  uint32_t code; /* GAL_VEB_OP_* */
  uint32_t tid;  /* executing thread id (< 1024) for the hashed ops */
  uint64_t arg;
  uint64_t arg2;
} gal_veb_op;

#define GAL_VEB_OP_INSERT 0             /* insert(arg) -> bool           veb.cuh:757 */
#define GAL_VEB_OP_INSERT_FORCE 1       /* insert_force_update(arg)      veb.cuh:775 */
#define GAL_VEB_OP_REMOVE 2             /* remove(arg) -> bool           veb.cuh:737 */
#define GAL_VEB_OP_QUERY 3              /* query(arg) -> bool            veb.cuh:824 */
#define GAL_VEB_OP_SUCCESSOR 4          /* successor(arg) -> id|~0       veb.cuh:836 */
#define GAL_VEB_OP_SUCCESSOR_THOROUGH 5 /* successor_thorough(arg)       veb.cuh:878 */
#define GAL_VEB_OP_LOCK_OFFSET 6        /* lock_offset(arg)              veb.cuh:918 */
#define GAL_VEB_OP_MALLOC_FIRST 7       /* malloc_first()                veb.cuh:979 */
#define GAL_VEB_OP_FIND_FIRST 8         /* find_first_valid_index()      veb.cuh:940 */
#define GAL_VEB_OP_FIND_RANDOM 9        /* find_random_valid_index()     veb.cuh:946 */
#define GAL_VEB_OP_MALLOC 10            /* malloc()                      veb.cuh:993 */
#define GAL_VEB_OP_GATHER 11            /* gather_multiple(arg)          veb.cuh:1160 */
#define GAL_VEB_OP_RETURN 12            /* return_multiple(arg, arg2)    veb.cuh:1198 */
#define GAL_VEB_OP_REPORT_FILL 13       /* set leaf bits                 veb.cuh:1052 */
/* The allocator's own searches (no reference counterpart; the reference's
 * allocator uses find_random_valid_index and malloc_first): valid on trees
 * whose upper layers are the OR of their children, i.e. trees changed only
 * by INSERT_FORCE and REMOVE. */
#define GAL_VEB_OP_FIND_AT_OR_AFTER 14  /* smallest set id >= arg, or ~0 */
#define GAL_VEB_OP_CLAIM_FIRST 15       /* remove and return the smallest set id, or ~0 */

/* Full tree over [0, universe) (reference veb_tree::generate_on_device). */
int gal_veb_create(uint64_t universe, uint64_t seed, gal_veb **out);
int gal_veb_destroy(gal_veb *v);
int gal_veb_num_layers(gal_veb *v);
uint64_t gal_veb_layer_words(gal_veb *v, int layer);
int gal_veb_dump(gal_veb *v, int layer, uint64_t *host_dst);
/* Run ops in order on one 1024-thread block; op i runs on thread ops[i].tid
 * and writes results[i]. d_ops/d_results are device buffers. */
int gal_veb_run_ops(gal_veb *v, const gal_veb_op *d_ops, uint64_t n, uint64_t *d_results, void *stream);

/* Replace the tree's contents: host_leaf holds the leaf layer's words (bit i
 * of word w = id 64w + i; no bit at or past the universe), and every upper
 * layer is rebuilt as the OR of its child words, the state insert_force_update
 * keeps. No reference counterpart (the reference fills a tree by inserts).
 * Synchronous. */
int gal_veb_load(gal_veb *v, const uint64_t *host_leaf, uint64_t words);
/* For each of n device queries x, d_out = the smallest set id >= x, or ~0
 * (the result GAL_VEB_OP_FIND_AT_OR_AFTER gives), on a tree whose upper
 * layers are the OR of their children and that nothing changes during the
 * call. staged = 1: each CTA first copies the tree's upper layers (as many
 * of the top layers as fit 48 KiB of shared memory) into shared memory and
 * answers its queries from there, with the leaf words read in aligned
 * 128-bit pairs; staged = 0: one thread per query reading every layer from
 * global memory (veb::find_at_or_after). No reference counterpart: the
 * reference answers one successor at a time (veb.cuh:836-916). */
int gal_veb_find_batch(gal_veb *v, const uint64_t *d_queries, uint64_t n, uint64_t *d_out, uint32_t staged,
                       void *stream);

/* Last CUDA error text recorded by this library (static storage). */
const char *gal_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* GALLATIN_GB300_H */

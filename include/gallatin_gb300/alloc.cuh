// Device allocator core: the three tiers of Gallatin's method on GB300.
//
//   slice tier    size <= max: a pinned block of the size's tree serves the
//                 request; multi-slice runs of 2..64 slices for sizes up to
//                 min*4096/2 (reference gallatin.cuh:1196-1217)
//   block tier    up to segment size: a whole block (gallatin.cuh:828-861)
//   segment tier  n contiguous segments (gallatin.cuh:790-826)
//
// The method is the reference's: segments tracked by vEB trees (the segment
// tree hands out the smallest free id, sub trees pick a hashed random start),
// segments formatted into power-of-two blocks of 4096 slices, a memory table
// (chunk_ids) that maps a pointer back to its segment's tree on free.
//
// The GB300 design differs in how a block hands out slices. The reference
// bumps a per-block counter and recycles a block only after all 4096 slices
// came back (block.cuh:245-281). Here each block carries a 4096-bit slice
// bitmap: a warp's same-class requests reserve capacity with one atomic on
// the block's meta word (live count + cursor + tree/state tag), then claim
// bits with fetch-and; frees return bits with fetch-or and release the
// reservation. Freed slices are reused while the block stays pinned, so a
// block is replaced only when it is full, and it is recycled to its
// segment's free-block bitmap when its last slice comes back. A replaced
// block that still holds slices is detached; once half of it has drained it
// is pinned again ahead of a fresh block, so long-lived allocations freed in
// random order do not strand the arena in half-empty blocks. Blocks of the
// largest tree serve one run length each (1, 2, 4 ... slices) for as long as
// they are out of their segment, so multi-slice runs never fragment. Every
// wait is bounded; exhausted budgets return nullptr and bump a device counter.
#ifndef GALLATIN_GB300_ALLOC_CUH
#define GALLATIN_GB300_ALLOC_CUH

#include <stdint.h>

#include "ptx.cuh"
#include "state.h"
#include "veb.cuh"

// Marks the paths taken once per block or segment change (slot replacement,
// the block and segment tiers). They are inlined by default: compiled out of
// line (-DGAL_COLD=__noinline__) they shrink the calling kernels and their
// build time by about ten times, but the calls cost the mixed workload 14 %
// and the plain 16 B workload 11 % on a GB300 (the hash table was level).
#ifndef GAL_COLD
#define GAL_COLD
#endif

namespace gal {

constexpr int kSliceAttempts = 4096;      // group attempts per slice request
constexpr int kClaimSteps = 256;          // fetch-and steps per reservation
constexpr int kRequestBlockAttempts = 512;
constexpr int kSegmentLockBit = 31;
// a pinned block past this many live slices is replaced ahead of time, so
// warps rarely find their slot's block full
constexpr uint32_t kRefillMark = GAL_BLOCK_SLICES * 7 / 8;
constexpr int kAdoptCandidates = 64;
// leader-to-group markers: the slot is full and no block can replace it;
// the slot cannot serve while another leader replaces its block
constexpr uint32_t kNoMemBlock = 0xFFFFFFFEu;
constexpr uint32_t kBusyBlock = 0xFFFFFFFDu;
// leader-to-group flag on the cursor: the slices were taken by cursor alone
constexpr uint32_t kFreshClaim = 1u << 31;

// which detached blocks request_block may pin again
enum { ADOPT_NONE = 0, ADOPT_ROOMY = 1, ADOPT_ANY = 2 };
enum { REPLACE_OK = 0, REPLACE_BUSY = 1, REPLACE_NOMEM = 2 };

enum { TIER_SLICE = 0, TIER_BLOCK = 1, TIER_SEGMENT = 2 };

struct size_class {
  int tier;
  uint32_t tree;   // slice tree (slice tier) or block tree (block tier)
  uint32_t count;  // slices per request (slice tier)
  uint64_t nseg;   // segments (segment tier)
};

// Smallest e with 2^e >= v, for v >= 1 (reference get_first_bit_bigger,
// alloc_utils.cuh:382-398).
__host__ __device__ __forceinline__ int ceil_log2(uint64_t v) {
#ifdef __CUDA_ARCH__
  return 63 - __clzll((long long)v) + (__popcll(v) != 1);
#else
  return 63 - __builtin_clzll(v) + (__builtin_popcountll(v) != 1);
#endif
}

// Size classing, identical to the reference's malloc dispatch
// (gallatin.cuh:1141-1147, 1196-1260).
__host__ __device__ __forceinline__ size_class classify(int min_shift, int num_trees, int block_shift_min,
                                                        int segment_shift, uint64_t size) {
  size_class sc;
  sc.tier = TIER_SLICE;
  sc.tree = 0;
  sc.count = 1;
  sc.nseg = 0;
  if (size < (1ull << min_shift)) return sc;
  const int cl = ceil_log2(size);
  const int tree = cl - min_shift;
  if (tree < num_trees) {
    sc.tree = (uint32_t)tree;
    return sc;
  }
  const int block_tree = cl - block_shift_min;
  if (block_tree < 0) {
    sc.tree = (uint32_t)(num_trees - 1);
    sc.count = 1u << (tree - (num_trees - 1));
    return sc;
  }
  if (block_tree < num_trees) {
    sc.tier = TIER_BLOCK;
    sc.tree = (uint32_t)block_tree;
    return sc;
  }
  sc.tier = TIER_SEGMENT;
  sc.nseg = ((size - 1) >> segment_shift) + 1;
  return sc;
}

__device__ __forceinline__ size_class classify(const gal_state_t *st, uint64_t size) {
  return classify(st->min_shift, st->num_trees, st->block_shift_min, st->segment_shift, size);
}

__device__ __forceinline__ uint32_t meta_live(uint64_t m) { return (uint32_t)m; }
__device__ __forceinline__ uint32_t meta_tree(uint64_t m) { return (uint32_t)(m >> GAL_META_TREE_SHIFT) & 0xFFu; }
__device__ __forceinline__ uint32_t meta_state(uint64_t m) { return (uint32_t)(m >> GAL_META_STATE_SHIFT) & 3u; }
__device__ __forceinline__ uint32_t meta_run(uint64_t m) { return (uint32_t)(m >> GAL_META_RUN_SHIFT) & 0xFu; }
__device__ __forceinline__ uint32_t meta_class(uint64_t m) { return meta_tree(m) + meta_run(m); }
__device__ __forceinline__ uint32_t meta_cursor(uint64_t m) { return (uint32_t)(m >> GAL_META_CURSOR_SHIFT); }
// tree, state and run fields together (bits 32-45)
__device__ __forceinline__ uint32_t meta_tag(uint64_t m) { return (uint32_t)(m >> GAL_META_TREE_SHIFT) & 0x3FFFu; }

__device__ __forceinline__ void count(const gal_state_t *st, int id) {
  atomicAdd(st->counters + id, 1ull);
}

__device__ __forceinline__ int block_index_shift(const gal_state_t *st) {
  return st->segment_shift - st->block_shift_min;
}

__device__ __forceinline__ char *block_address(const gal_state_t *st, uint64_t b, uint32_t t) {
  const int bis = block_index_shift(st);
  const uint64_t seg = b >> bis;
  const uint64_t i = b & ((1ull << bis) - 1);
  return st->memory + (seg << st->segment_shift) + (i << (st->block_shift_min + (int)t));
}

// Aligned runs of c (a power of two <= 64) free bits: bit j is set when bits
// j..j+c-1 are all set and j is a multiple of c.
__device__ __forceinline__ uint64_t run_starts(uint64_t a, uint32_t c) {
  if (c == 1) return a;
  if (c >= 64) return (a == ~0ull) ? 1ull : 0ull;
  uint64_t x = a;
  for (uint32_t s = 1; s < c; s <<= 1) x &= x >> s;
  return x & (~0ull / ((1ull << c) - 1));
}

__device__ __forceinline__ uint64_t expand_runs(uint64_t starts, uint32_t c) {
  if (c >= 64) return starts ? ~0ull : 0ull;
  return starts * ((1ull << c) - 1);
}

__device__ __forceinline__ uint64_t lowest_bits(uint64_t x, uint32_t k) {
  uint64_t out = 0;
  for (uint32_t i = 0; i < k && x; ++i) {
    uint64_t low = x & (~x + 1);
    out |= low;
    x ^= low;
  }
  return out;
}

__device__ __forceinline__ void backoff(int attempt) {
  int ns = 32 << ((attempt >> 4) < 5 ? (attempt >> 4) : 5);
  __nanosleep(ns);
}

// ---- tree searches ------------------------------------------------------
//
// The allocator's searches of its own trees. By default they are the
// reference's operations (successor_thorough, find_random_valid_index,
// malloc_first), which read one word per load. With -DGAL_PAIR_SEARCH they
// are veb::find_at_or_after and its relatives, which read the leaf in
// aligned 128-bit word pairs and merge the query with the first scan. Both
// give the same answers on a quiescent tree (tests/test_veb_gpu.py checks
// the pair searches against a brute-force set model), but under contention
// the pair searches made the exact-capacity and mixed-tier tests see more
// NULLs (2-4 of 16 runs short, against none in 108 runs with the default),
// for a reason not yet found, so they stay off.
__device__ __forceinline__ uint64_t tree_at_or_after(const gal_veb_t *t, uint64_t x) {
#ifdef GAL_PAIR_SEARCH
  return veb::find_at_or_after(t, x);
#else
  if (x >= t->universe) return veb::kFail;
  if (veb::query(t, x)) return x;
  return veb::successor_thorough(t, x);
#endif
}

__device__ __forceinline__ bool veb_maybe_nonempty(const gal_veb_t *v) {
  for (uint64_t w = 0; w < v->layer_words[0]; ++w)
    if (ptx::ld_relaxed(v->bits[0] + w)) return true;
  return false;
}

// A tree whose top layer reads empty twice, 2 us apart. The reference's
// searches make 15 attempts of several dependent loads each before they
// report an empty tree (about 100 loads for a block replacement that finds
// neither a sub-tree segment nor a free segment, the common case once the
// arena is full); the second look covers an insert whose upper-layer bits are
// still on their way up, which those attempts rode out by taking long.
__device__ inline bool veb_seems_empty(const gal_veb_t *v) {
  if (veb_maybe_nonempty(v)) return false;
  __nanosleep(2000);
  return !veb_maybe_nonempty(v);
}

__device__ __forceinline__ uint64_t tree_hashed(const gal_veb_t *t, uint64_t tid) {
#ifdef GAL_PAIR_SEARCH
  return veb::find_hashed(t, tid);
#else
  if (veb_seems_empty(t)) return veb::kFail;
  return veb::find_random_valid_index(t, tid);
#endif
}

__device__ __forceinline__ uint64_t tree_claim_first(const gal_veb_t *t) {
#ifdef GAL_PAIR_SEARCH
  return veb::claim_first(t);
#else
  if (veb_seems_empty(t)) return veb::kFail;
  return veb::malloc_first(t);
#endif
}

// ---- locks (bounded) -----------------------------------------------------

__device__ __forceinline__ bool try_lock(const gal_state_t *st, int bit) {
  return (atomicOr(st->locks, 1u << bit) & (1u << bit)) == 0;
}

__device__ __forceinline__ void unlock(const gal_state_t *st, int bit) {
  __threadfence();
  atomicAnd(st->locks, ~(1u << bit));
}

// ---- segments ------------------------------------------------------------

// A segment belongs in sub tree t exactly while it is formatted for t and has
// a free block. Callers that change either fact call this afterwards: it
// applies the membership it observes and re-reads until the observation is
// stable, so the last change always wins. Under contention a segment can be
// listed without a free block for a moment (searches then fail on it and
// sync it again); it is never left unlisted while it has a free block.
// The fences around each apply make "last" mean what it says: a fact change
// is ordered before its author's membership update, and a membership update
// that lands after another one (they are read-modify-writes of one word) is
// ordered before its author's re-read, which therefore sees the other
// author's fact change. Without them the re-read could return a fact older
// than a retire whose remove it had just overwritten, and leave a retired
// segment listed.
__device__ __forceinline__ bool seg_listed_for(const gal_state_t *st, uint32_t t, uint64_t seg) {
  return ptx::ld_relaxed(st->chunk_ids + seg) == t && ptx::ld_relaxed(st->seg_avail + seg) > 0;
}

__device__ inline void sub_tree_sync(const gal_state_t *st, uint32_t t, uint64_t seg) {
  const gal_veb_t *sub = &st->sub_trees[t];
  bool want = seg_listed_for(st, t, seg);
  for (int i = 0; i < 8; ++i) {
    ptx::fence_acq_rel();
    if (want) {
      veb::insert_force_update(sub, seg);
    } else {
      veb::remove(sub, seg);
    }
    ptx::fence_acq_rel();
    const bool now = seg_listed_for(st, t, seg);
    if (now == want) return;
    want = now;
  }
}

__device__ inline void try_retire_segment(const gal_state_t *st, uint64_t seg, uint32_t t, int32_t bps_t) {
  if (ptx::cas_acq_rel(st->seg_avail + seg, bps_t, (int32_t)GAL_SEG_GATE) != bps_t) return;
  sub_tree_sync(st, t, seg);
  unsigned short prev = atomicCAS((unsigned short *)(st->chunk_ids + seg), (unsigned short)t,
                                  (unsigned short)GAL_FREE_SEGMENT);
  if (prev != (unsigned short)t) count(st, GAL_CTR_CORRUPT);
  __threadfence();
  veb::insert_force_update(&st->segment_tree, seg);
  count(st, GAL_CTR_SEGMENT_RETIRE);
}

// Add one free block to a segment's count and act on the transitions:
// 0 -> 1 makes the segment findable again, all-free retires it.
__device__ inline void seg_avail_add_one(const gal_state_t *st, uint64_t seg) {
  const int32_t now = ptx::atom_add_release(st->seg_avail + seg, 1) + 1;
  if (now <= 0) return;
  const uint32_t t = ptx::ld_relaxed(st->chunk_ids + seg);
  if (t >= (uint32_t)st->num_trees) return;
  const int32_t bps_t = (int32_t)(st->blocks_per_segment >> t);
  if (now == bps_t) {
    try_retire_segment(st, seg, t, bps_t);
  } else if (now == 1) {
    sub_tree_sync(st, t, seg);
  }
}

// Format the smallest free segment for tree t. Callers hold tree t's lock
// when a segment of t has several blocks, so that concurrent requests do not
// each format one; every step is atomic on its own.
__device__ inline uint64_t attach_segment(const gal_state_t *st, uint32_t t) {
  const uint64_t seg = tree_claim_first(&st->segment_tree);  // smallest free id (reference malloc_first)
  if (seg == veb::kFail) return veb::kFail;
  unsigned short prev = atomicCAS((unsigned short *)(st->chunk_ids + seg), (unsigned short)GAL_FREE_SEGMENT,
                                  (unsigned short)t);
  if (prev != (unsigned short)GAL_FREE_SEGMENT) {
    count(st, GAL_CTR_CORRUPT);
    return veb::kFail;
  }
  const uint32_t bps_t = st->blocks_per_segment >> t;
  uint64_t *words = st->seg_block_bits + seg * st->seg_block_words;
  for (uint32_t w = 0; w < st->seg_block_words; ++w) {
    const uint32_t lo = w * 64;
    uint64_t v = 0;
    if (bps_t >= lo + 64) v = ~0ull;
    else if (bps_t > lo) v = (1ull << (bps_t - lo)) - 1;
    ptx::st_relaxed(words + w, v);
  }
  ptx::atom_add_release(st->seg_avail + seg, (int32_t)bps_t - (int32_t)GAL_SEG_GATE);
  sub_tree_sync(st, t, seg);
  count(st, GAL_CTR_SEGMENT_ATTACH);
  return seg;
}

// Take one free block out of segment `seg` (formatted for t). Returns its
// global block id, exclusively owned and in state FREE, or GAL_EMPTY_BLOCK.
__device__ inline uint32_t take_block(const gal_state_t *st, uint64_t seg, uint32_t t) {
  const int32_t before = ptx::atom_add_acquire(st->seg_avail + seg, -1);
  if (before <= 0) {
    seg_avail_add_one(st, seg);
    sub_tree_sync(st, t, seg);
    return GAL_EMPTY_BLOCK;
  }
  if (ptx::ld_relaxed(st->chunk_ids + seg) != t) {
    seg_avail_add_one(st, seg);
    sub_tree_sync(st, t, seg);
    return GAL_EMPTY_BLOCK;
  }
  if (before == 1) sub_tree_sync(st, t, seg);
  uint64_t *words = st->seg_block_bits + seg * st->seg_block_words;
  const int bis = block_index_shift(st);
  // the segment's words are read in aligned pairs (seg_block_words is even)
  for (int pass = 0; pass < 64; ++pass) {
    for (uint32_t w = 0; w < st->seg_block_words; w += 2) {
      uint64_t pair[2];
      ptx::ld_relaxed_v2(words + w, pair[0], pair[1]);
      for (uint32_t h = 0; h < 2; ++h) {
        uint64_t v = pair[h];
        while (v) {
          const uint64_t bit = v & (~v + 1);
          const uint64_t old = ptx::atom_and_acquire(words + w + h, ~bit);
          if (old & bit) return (uint32_t)((seg << bis) + (w + h) * 64 + (uint64_t)(__ffsll((long long)bit) - 1));
          v = old & ~bit;
        }
      }
    }
  }
  count(st, GAL_CTR_CORRUPT);
  seg_avail_add_one(st, seg);
  return GAL_EMPTY_BLOCK;
}

// A block or segment went back to its pool: the no-memory hints of every
// class are out of date.
__device__ __forceinline__ void clear_nomem(const gal_state_t *st) {
  if (ptx::ld_relaxed(st->nomem)) atomicExch(st->nomem, 0u);
}

// Give a retired block back to its segment's free-block bitmap.
__device__ inline void return_block_to_segment(const gal_state_t *st, uint64_t b) {
  const int bis = block_index_shift(st);
  const uint64_t seg = b >> bis;
  const uint64_t i = b & ((1ull << bis) - 1);
  ptx::red_or_relaxed(st->seg_block_bits + seg * st->seg_block_words + (i >> 6), 1ull << (i & 63));
  seg_avail_add_one(st, seg);  // release add orders the bit before the count
  count(st, GAL_CTR_BLOCK_RETIRE);
  clear_nomem(st);
}

// A block belongs in class k's adoptable tree exactly while it is DETACHED,
// serves class k and has room (live below a full block: a block of the
// largest tree holds whole runs, so that is room for one more run), and in
// class k's roomy tree while in addition its live count is at most
// GAL_ROOMY_MARK (same apply-then-confirm discipline as sub_tree_sync: the
// last change to the facts is always applied). Full detached blocks stay off
// the adoptable tree, so an adopter's bounded scan does not spend itself on
// them; the free that gives such a block room lists it again.
__device__ __forceinline__ bool adopt_listed(uint64_t m, uint32_t k, bool roomy) {
  return meta_state(m) == GAL_STATE_DETACHED && meta_class(m) == k && meta_live(m) < GAL_BLOCK_SLICES &&
         (!roomy || meta_live(m) <= GAL_ROOMY_MARK);
}

__device__ inline void adopt_sync(const gal_state_t *st, uint32_t k, uint64_t b, bool roomy) {
  const gal_veb_t *at = roomy ? &st->roomy_trees[k] : &st->adopt_trees[k];
  bool want = adopt_listed(ptx::ld_relaxed(st->block_meta + b), k, roomy);
  for (int i = 0; i < 8; ++i) {
    if (want) {
      veb::insert_force_update(at, b);
    } else {
      veb::remove(at, b);
    }
    const bool now = adopt_listed(ptx::ld_relaxed(st->block_meta + b), k, roomy);
    if (now == want) return;
    want = now;
  }
}

__device__ __forceinline__ void adopt_sync_both(const gal_state_t *st, uint32_t k, uint64_t b) {
  adopt_sync(st, k, b, false);
  adopt_sync(st, k, b, true);
}

// A DETACHED block whose live count reached zero, or a block-tier (WHOLE)
// block whose allocation was freed, goes back to its segment.
__device__ inline void try_retire_block(const gal_state_t *st, uint64_t b) {
  uint64_t *mp = st->block_meta + b;
  uint64_t m = ptx::ld_relaxed(mp);
  for (int i = 0; i < 64; ++i) {
    const uint32_t state = meta_state(m);
    if ((state != GAL_STATE_DETACHED && state != GAL_STATE_WHOLE) || meta_live(m) != 0) return;
    const uint64_t nm = m - ((uint64_t)state << GAL_META_STATE_SHIFT);
    const uint64_t r = ptx::cas_acq_rel(mp, m, nm);
    if (r == m) {
      if (state == GAL_STATE_DETACHED) adopt_sync_both(st, meta_class(m), b);
      return_block_to_segment(st, b);
      return;
    }
    m = r;
  }
}

// Give back n slices of block b's live count and act on the transitions.
// `ordered`: the caller has already fenced (free_slice), so the add itself
// can be relaxed.
__device__ inline void after_release(const gal_state_t *st, uint64_t b, uint32_t n, uint64_t old) {
  const uint32_t live = meta_live(old);
  if (live == n) {
    try_retire_block(st, b);
    return;
  }
  if (meta_state(old) != GAL_STATE_DETACHED) return;
  // a full detached block got room (also the undo of a reservation that
  // found the block already detached): list it as adoptable again
  if (live >= GAL_BLOCK_SLICES && live - n < GAL_BLOCK_SLICES) adopt_sync(st, meta_class(old), b, false);
  if (live > GAL_ROOMY_MARK && live - n <= GAL_ROOMY_MARK) adopt_sync(st, meta_class(old), b, true);
}

__device__ __forceinline__ void release_live(const gal_state_t *st, uint64_t b, uint32_t n, bool ordered = false) {
  const uint64_t delta = (uint64_t)(-(int64_t)n);
  const uint64_t old =
      ordered ? ptx::atom_add_relaxed(st->block_meta + b, delta) : ptx::atom_add_release(st->block_meta + b, delta);
  // a PINNED block has nothing to do; DETACHED and WHOLE ones may retire or
  // become roomy
  if (meta_state(old) >= GAL_STATE_DETACHED) after_release(st, b, n, old);
}

// Move a block this thread owns from FREE to `state`, formatted for tree t
// and run length 2^r, adding `live` to its live count, with the cursor at 0
// and the fresh flag as given. (A stale reservation may still add to live and
// cursor meanwhile; its undo gives back live only, so it can only move the
// cursor past positions that then stay free for a later pass.)
__device__ __forceinline__ void own_block(const gal_state_t *st, uint64_t b, uint32_t t, uint32_t r,
                                          uint32_t state, uint32_t live, bool fresh = false) {
  const uint64_t m = ptx::ld_relaxed(st->block_meta + b);
  const int64_t dstate = (int64_t)state - (int64_t)meta_state(m);
  const int64_t dtree = (int64_t)t - (int64_t)meta_tree(m);
  const int64_t drun = (int64_t)r - (int64_t)meta_run(m);
  const uint64_t dcursor = (uint64_t)(0x10000u - meta_cursor(m)) << GAL_META_CURSOR_SHIFT;  // wraps to 0
  const uint64_t delta = (uint64_t)(dstate * (1ll << GAL_META_STATE_SHIFT)) +
                         (uint64_t)(dtree * (1ll << GAL_META_TREE_SHIFT)) +
                         (uint64_t)(drun * (1ll << GAL_META_RUN_SHIFT)) - (m & GAL_META_REUSED_BIT) -
                         (m & GAL_META_FRESH_BIT) + (fresh ? GAL_META_FRESH_BIT : 0) + dcursor + (uint64_t)live;
  ptx::atom_add_release(st->block_meta + b, delta);
}

__device__ __forceinline__ uint64_t mix_tid(uint64_t tid, int attempt) {
  return attempt == 0 ? tid : murmur64a_u64(tid, (uint64_t)attempt);
}

// Pin again a DETACHED block of class k (tree t, run length c slices): from
// the roomy tree (live <= GAL_ROOMY_MARK), or from the adoptable tree any
// block with room for one more run. The block keeps its live slices and its
// bitmap. Candidates are visited from a hashed start so that concurrent
// adopters spread out.
__device__ inline uint32_t adopt_block(const gal_state_t *st, uint32_t k, uint32_t c, uint64_t tid, bool roomy) {
  const gal_veb_t *at = roomy ? &st->roomy_trees[k] : &st->adopt_trees[k];
  if (!veb_maybe_nonempty(at)) return GAL_EMPTY_BLOCK;
  const uint64_t start = murmur64a_u64(tid, at->seed) % at->universe;
  uint64_t cand = tree_at_or_after(at, start);
  bool wrapped = false;
  for (int n = 0; n < kAdoptCandidates; ++n) {
    if (cand == veb::kFail) {
      if (wrapped) break;
      wrapped = true;
      cand = tree_at_or_after(at, 0);
      if (cand == veb::kFail) break;
    }
    uint64_t m = ptx::ld_relaxed(st->block_meta + cand);
    for (int i = 0; i < 8; ++i) {
      if (!adopt_listed(m, k, roomy) || meta_live(m) + c > GAL_BLOCK_SLICES) break;
      const uint64_t nm =
          ((m - ((uint64_t)(GAL_STATE_DETACHED - GAL_STATE_PINNED) << GAL_META_STATE_SHIFT)) | GAL_META_REUSED_BIT) &
          ~GAL_META_FRESH_BIT;
      const uint64_t r = ptx::cas_acq_rel(st->block_meta + cand, m, nm);
      if (r == m) {
        adopt_sync_both(st, k, cand);
        count(st, roomy ? GAL_CTR_ADOPT_ROOMY : GAL_CTR_ADOPT);
        return (uint32_t)cand;
      }
      m = r;
    }
    if (!adopt_listed(m, k, roomy)) adopt_sync(st, k, cand, roomy);
    cand = tree_at_or_after(at, cand + 1);
  }
  return GAL_EMPTY_BLOCK;
}

// A block for slot class k (tree t, run length c): with adopt_mode >=
// ADOPT_ROOMY first a detached block of the class that drained to half or
// less; then a FREE block from a segment already formatted for t or from a
// newly attached one; with ADOPT_ANY, when the arena has neither, a detached
// block with any room. An adopted block is already PINNED (*adopted = true).
// GAL_EMPTY_BLOCK when nothing can be had.
__device__ inline GAL_COLD uint32_t request_block(const gal_state_t *st, uint32_t t, uint32_t k, uint32_t c, uint64_t tid,
                                         int adopt_mode, bool *adopted) {
  *adopted = false;
  if (adopt_mode >= ADOPT_ROOMY) {
    const uint32_t b = adopt_block(st, k, c, tid, true);
    if (b != GAL_EMPTY_BLOCK) {
      *adopted = true;
      return b;
    }
  }
  const gal_veb_t *sub = &st->sub_trees[t];
  int a = 0;
  for (; a < kRequestBlockAttempts; ++a) {
    uint64_t seg = tree_hashed(sub, mix_tid(tid, a));
    if (seg == veb::kFail) {
      // a segment of one block serves exactly one request: no lock needed
      const bool solo = (st->blocks_per_segment >> t) == 1;
      if (!solo && !try_lock(st, (int)t)) {
        backoff(a);
        continue;
      }
      seg = attach_segment(st, t);
      if (!solo) unlock(st, (int)t);
      if (seg == veb::kFail) {
        if (tree_at_or_after(sub, 0) != veb::kFail) continue;
        break;  // no formatted segment with a free block, no free segment
      }
    }
    const uint32_t b = take_block(st, seg, t);
    if (b != GAL_EMPTY_BLOCK) return b;
  }
  if (a == kRequestBlockAttempts) count(st, GAL_CTR_TIMEOUT);
  if (adopt_mode == ADOPT_ANY) {
    const uint32_t b = adopt_block(st, k, c, tid, false);
    *adopted = b != GAL_EMPTY_BLOCK;
    return b;
  }
  return GAL_EMPTY_BLOCK;
}

// ---- pinned blocks -------------------------------------------------------

// The bitmap of a block that comes out of its segment is not rewritten: it
// starts all ones at creation, slices only ever leave it by claims and come
// back by frees, and a block-tier allocation leaves it alone, so the bitmap
// of a FREE block is all ones once every free in flight has landed. A free
// still in flight holds a 0 that nobody can claim until it turns to 1; that
// is what lets free_slice return bits and live count in either order.
// The block holds no slice here, so any 0 bit is such a free: with none, the
// block is pinned fresh and its first pass hands out slices by cursor (each
// group still fetch-ands its bits: see malloc_slice).
__device__ inline void pin_block(const gal_state_t *st, uint64_t b, uint32_t t, uint32_t r) {
  const ulonglong2 *bits = reinterpret_cast<const ulonglong2 *>(st->block_bits + (b << 6));
  uint64_t all = ~0ull;
  for (int i = 0; i < 32; ++i) {
    const ulonglong2 v = __ldcg(bits + i);
    all &= v.x & v.y;
  }
  own_block(st, b, t, r, GAL_STATE_PINNED, 0, all == ~0ull);
  count(st, GAL_CTR_BLOCK_PINS);
  count(st, GAL_CTR_TREE_PINS + (int)t);
}

__device__ inline void detach_block(const gal_state_t *st, uint64_t b) {
  const uint64_t old = ptx::atom_add_release(
      st->block_meta + b, (uint64_t)(GAL_STATE_DETACHED - GAL_STATE_PINNED) << GAL_META_STATE_SHIFT);
  if (meta_live(old) == 0) {
    try_retire_block(st, b);
  } else {
    adopt_sync(st, meta_class(old), b, false);
    // a release that crossed the mark before the detach could not list it
    if (meta_live(old) <= GAL_ROOMY_MARK) adopt_sync(st, meta_class(old), b, true);
  }
}

// Replace the block a slot holds (`seen`, without the REPLACING flag) by
// another pinned one. Only the thread whose CAS sets REPLACING does the work;
// REPLACE_NOMEM when request_block found nothing (the slot is left as seen).
__device__ inline GAL_COLD int replace_slot(const gal_state_t *st, uint64_t *slot, uint64_t seen, uint32_t t, uint32_t r,
                                   int adopt_mode, uint32_t *out) {
  // the hashed search starts come from the thread id, read here rather than
  // carried through the claim loop
  const uint64_t tid = veb::thread_tid();
  *out = GAL_EMPTY_BLOCK;
  if (atomicCAS((unsigned long long *)slot, seen, seen | GAL_SLOT_REPLACING) != seen) return REPLACE_BUSY;
  bool adopted = false;
  uint32_t nb = request_block(st, t, t + r, 1u << r, tid, adopt_mode, &adopted);
  const uint32_t kbit = 1u << (t + r);
  if (nb == GAL_EMPTY_BLOCK && adopt_mode == ADOPT_ANY) {
    // before the class is declared out of memory: a reservation that found
    // its block already detached is undone one round trip later, and until
    // then that block can look full to an adopter. Look once more.
    __nanosleep(2000);
    nb = adopt_block(st, t + r, 1u << r, tid, false);
    adopted = nb != GAL_EMPTY_BLOCK;
  }
  if (nb == GAL_EMPTY_BLOCK) {
    ptx::st_release(slot, seen);
    if (adopt_mode == ADOPT_ANY && !(ptx::ld_relaxed(st->nomem) & kbit)) atomicOr(st->nomem, kbit);
    return REPLACE_NOMEM;
  }
  if (ptx::ld_relaxed(st->nomem) & kbit) atomicAnd(st->nomem, ~kbit);
  if (!adopted) pin_block(st, nb, t, r);
  ptx::st_release(slot, (uint64_t)nb);
  if ((uint32_t)seen != GAL_EMPTY_BLOCK) detach_block(st, (uint32_t)seen);
  *out = nb;
  return REPLACE_OK;
}

// ---- slice tier ----------------------------------------------------------

// Lanes of the tile of `width` lanes (8, 16 or 32) that holds this lane.
__device__ __forceinline__ uint32_t tile_mask(uint32_t width) {
  if (width >= 32) return 0xffffffffu;
  const uint32_t lane = ptx::laneid();
  return ((1u << width) - 1) << (lane & ~(width - 1));
}

// Warp-aggregated slice allocation of one run of 2^r slices of tree t. Lanes
// asking for the same class form one group; its leader reserves the group's
// total with one atomic on the pinned block's meta word and claims bits with
// fetch-and. Once a replacement finds no block in the arena for the class
// (or the group meets a slot being replaced while the last replacement for
// the class found none), the group asks for no more blocks: each further slot
// it finds full or empty is a strike, and after a strike on every slot the
// arena cannot serve the class now (nullptr).
__device__ __forceinline__ void *malloc_slice(const gal_state_t *st, uint32_t t, uint32_t r, uint32_t width = 32) {
  const uint32_t c = 1u << r;
  const uint32_t k = t + r;
  const uint32_t active = __activemask();
  const uint32_t peers = __match_any_sync(active, k) & tile_mask(width);
  const uint32_t lane = ptx::laneid();
  const uint32_t lt = ptx::lanemask_lt();
  const uint32_t nslots = st->slot_count[k];
  // (integer remainders by a run-time count are long sequences: skipped when
  // the value is already in range, the common case)
  const uint32_t sm = ptx::smid();
  const uint32_t slot0 = sm < nslots ? sm : sm % nslots;
  uint64_t *const slots = st->slots + st->slot_offset[k];
  // tree, state and run fields of a block pinned for this class
  const uint32_t tag = t | (GAL_STATE_PINNED << (GAL_META_STATE_SHIFT - 32)) | (r << (GAL_META_RUN_SHIFT - 32));
  void *result = nullptr;
  bool done = false;
  uint32_t hops = 0;     // slots passed over while another leader replaced their block
  uint32_t strikes = 0;  // slots found full or empty once the arena had no block for the class
  uint32_t missed = 0;   // slot index (before the remainder) of the last visit outside strike mode
  bool last_pass = false;  // the strikes were reset once before giving up
  for (int attempt = 0; attempt < kSliceAttempts; ++attempt) {
    const uint32_t grp = __ballot_sync(peers, !done);
    if (grp == 0) break;
    if (done) continue;
    const int leader = __ffs((int)grp) - 1;
    const uint32_t g_n = __popc(grp);
    const uint32_t g_rank = __popc(grp & lt);
    const uint32_t need = g_n * c;
    // after a miss each other slot is visited once, in order from the
    // missed one, so a strike on every slot means every slot was seen full
    // or empty. (The miss is not always at slot0: after busy hops, or eight
    // attempts on one slot, a group has moved on, and counting from slot0
    // left slot0 unvisited.)
    uint32_t slot_i;
    if (strikes) {
      slot_i = missed + strikes;
    } else {
      slot_i = slot0 + (uint32_t)(attempt >> 3) + hops;
      missed = slot_i;
    }
    if (slot_i >= nslots) slot_i %= nslots;
    uint64_t *const slot = slots + slot_i;

    uint32_t b = GAL_EMPTY_BLOCK;
    uint32_t cursor = 0;
    uint32_t take = 0;  // runs this attempt serves: the group, or what still fits
    uint32_t lost = 0;  // fresh claim: group ranks whose run a bitmap claim took first
    bool nomem = false;
    bool busy = false;
    bool refill = false;
    if (lane == (uint32_t)leader) {
      const uint64_t sv = ptx::ld_acquire(slot);
      const bool replacing = (sv & GAL_SLOT_REPLACING) != 0;
      b = (uint32_t)sv;
      if (b == GAL_EMPTY_BLOCK) {
        if (strikes) {
          nomem = true;  // the arena had no block for the class: do not ask again
        } else if (!replacing) {
          count(st, GAL_CTR_REPLACE_EMPTY);
          nomem = replace_slot(st, slot, sv, t, r, ADOPT_ANY, &b) == REPLACE_NOMEM;
        } else {
          count(st, GAL_CTR_SLOT_BUSY);
          // the last pass passes over busy slots until it can replace one
          nomem = !last_pass && ((ptx::ld_relaxed(st->nomem) >> k) & 1u);
          busy = !nomem;
        }
      }
      if (b != GAL_EMPTY_BLOCK) {
        // the block stays usable while another leader replaces it
        uint64_t m = ptx::atom_add_acquire(st->block_meta + b, ((uint64_t)need << GAL_META_CURSOR_SHIFT) | need);
        take = g_n;
        if (meta_tag(m) != tag) {
          release_live(st, b, need);
          count(st, GAL_CTR_STALE_SLOT);
          take = 0;
        } else if (meta_live(m) + need > GAL_BLOCK_SLICES) {
          // full for the whole group: undo, then reserve what still fits
          release_live(st, b, need);
          const uint32_t room = meta_live(m) < GAL_BLOCK_SLICES ? GAL_BLOCK_SLICES - meta_live(m) : 0;
          take = room / c < g_n ? room / c : g_n;
          if (take > 0) {
            const uint32_t part = take * c;
            m = ptx::atom_add_acquire(st->block_meta + b, ((uint64_t)part << GAL_META_CURSOR_SHIFT) | part);
            if (meta_tag(m) != tag || meta_live(m) + part > GAL_BLOCK_SLICES) {
              release_live(st, b, part);
              take = 0;
            }
          }
          if (take == 0) {
            if (strikes) {
              // the arena had no block for the class: do not ask again. But a
              // block can look full only because another group's reservation
              // on it is pending and about to be undone (two groups after the
              // last slices can each see the other's): look again, and strike
              // only a block with no room; one with room is tried again (in
              // strike mode the slot index does not move)
              const uint64_t again = ptx::ld_relaxed(st->block_meta + b);
              if (meta_tag(again) == tag && meta_live(again) + c <= GAL_BLOCK_SLICES) {
                busy = true;
              } else {
                nomem = true;
              }
            } else if (!replacing) {
              count(st, GAL_CTR_REPLACE_FULL);
              uint32_t nb;
              nomem = replace_slot(st, slot, (uint64_t)b, t, r, ADOPT_ANY, &nb) == REPLACE_NOMEM;
            } else {
              count(st, GAL_CTR_SLOT_BUSY);
              nomem = !last_pass && ((ptx::ld_relaxed(st->nomem) >> k) & 1u);
              busy = !nomem;
            }
          }
        } else if (!replacing && !strikes && meta_live(m) + need > kRefillMark) {
          refill = true;  // swap in another block once this group is served
        }
        if (take > 0) {
          cursor = meta_cursor(m);
          const uint32_t span = take * c;
          if ((m & GAL_META_FRESH_BIT) && cursor + span <= GAL_BLOCK_SLICES) {
            // first pass of a fresh block: no other fresh claim gets
            // [cursor, cursor + span), but a leader past the first pass
            // claims from the bitmap and may reach these bits before this
            // group clears them, so the bitmap decides: a run whose bits
            // were already taken is lost to this group (what of it this
            // fetch-and cleared goes back) and its lane tries again
            uint64_t *const fbits = st->block_bits + ((uint64_t)b << 6);
            for (uint32_t pos = cursor; pos < cursor + span;) {
              const uint32_t lo = pos & 63;
              const uint32_t n = 64 - lo < cursor + span - pos ? 64 - lo : cursor + span - pos;
              const uint64_t mask = (n >= 64 ? ~0ull : ((1ull << n) - 1)) << lo;
              const uint64_t old = ptx::atom_and_acquire(fbits + (pos >> 6), ~mask);
              if ((old & mask) != mask) {
                const uint64_t run = (c >= 64 ? ~0ull : ((1ull << c) - 1));
                for (uint32_t q = pos; q < pos + n; q += c) {
                  const uint64_t rm = run << (q & 63);
                  if ((old & rm) == rm) continue;
                  lost |= 1u << ((q - cursor) / c);
                  if (old & rm) ptx::red_or_relaxed(fbits + (pos >> 6), old & rm);
                }
              }
              pos += n;
            }
            if (lost) {
              release_live(st, b, (uint32_t)__popc(lost) * c);
              count(st, GAL_CTR_CLAIM_SHORT);
            }
            cursor |= kFreshClaim;
          } else {
            // past the first pass: the cursor must not look fresh after it wraps
            if (m & GAL_META_FRESH_BIT) ptx::red_and_relaxed(st->block_meta + b, ~GAL_META_FRESH_BIT);
            // Where the search starts. Allocations that live briefly come back
            // roughly in the order they went out, so the slices after the
            // cursor are the oldest and mostly free, and claiming them in
            // order keeps a block's live bytes together. A block more than
            // half live holds allocations that stay, freed in any order: the
            // words after the cursor are the ones just handed out and still
            // full (on the batching stream a claim walked 11 words on
            // average), so such a block, and one pinned again after a detach
            // (scattered by definition), starts each search at a hashed word.
            // The mark sits at half a block because a block that switches
            // between the two orders often (marks of 512 or 1024) loses
            // both: hashed claims punch holes ahead of the cursor.
            if ((m & GAL_META_REUSED_BIT) || meta_live(m) > GAL_ROOMY_MARK) cursor *= 0x9E3779B1u;
            cursor &= GAL_BLOCK_SLICES - 1;
          }
        } else {
          b = GAL_EMPTY_BLOCK;
        }
      }
      if (nomem) {
        count(st, GAL_CTR_NOMEM);
        b = kNoMemBlock;  // b was empty: nothing to serve from this attempt
      } else if (busy) {
        // try the next slot now; wait only after passing over all of them
        if ((hops + 1) % nslots == 0) backoff(attempt);
        b = kBusyBlock;
      }
    }
    b = __shfl_sync(grp, b, leader);
    cursor = __shfl_sync(grp, cursor, leader);
    if (b == kNoMemBlock) {
      if (++strikes >= nslots) {
        // a strike looks only at pinned blocks. A block detached with room
        // after the replacement that found nothing is pinned by nobody once
        // every group strikes, so before giving up the group makes one more
        // pass that starts as a normal one (its next full or empty slot is
        // replaced, adopting such a block)
        if (last_pass) {
          done = true;
        } else {
          last_pass = true;
          strikes = 0;
        }
      }
      continue;
    }
    if (b == kBusyBlock) {
      ++hops;
      continue;
    }
    if (b == GAL_EMPTY_BLOCK) continue;
    take = __shfl_sync(grp, take, leader);
    if (cursor & kFreshClaim) {  // the leader already holds these slices
      lost = __shfl_sync(grp, lost, leader);
      if (g_rank < take && !((lost >> g_rank) & 1u)) {
        const uint64_t slice = (cursor & ~kFreshClaim) + g_rank * c;
        result = block_address(st, b, t) + (slice << (st->min_shift + (int)t));
        done = true;
      }
      if (refill && lane == (uint32_t)leader) {
        count(st, GAL_CTR_REPLACE_REFILL);
        uint32_t nb;
        replace_slot(st, slot, (uint64_t)b, t, r, ADOPT_ROOMY, &nb);  // no nearly-full blocks
      }
      continue;
    }

    uint64_t *const bits = st->block_bits + ((uint64_t)b << 6);
    int my_slice = -1;
    uint32_t acc = 0;
    // leader-private search state: word, and what is known free in it
    uint32_t w = cursor >> 6;
    uint32_t lo = ((cursor & 63) + c - 1) & ~(c - 1);
    uint64_t avail = lo >= 64 ? 0ull : (~0ull << lo);
    // avail is still a whole range [lo, 64) (nothing learned about the word
    // yet): its lowest runs are its first (take - acc) * c bits, taken at
    // once instead of one run at a time (a warp's group of 32 single slices
    // spent 32 loop turns here)
    bool whole = true;
    for (int step = 0; step < kClaimSteps && acc < take; ++step) {
      uint64_t got = 0;
      uint32_t gw = w;
      if (lane == (uint32_t)leader) {
        uint64_t pick;
        if (whole) {
          const uint32_t from = avail ? (uint32_t)(__ffsll((long long)avail) - 1) : 64u;
          const uint32_t span = (take - acc) * c;
          pick = run_starts(span >= 64 - from ? avail : (((1ull << span) - 1) << from), c);
        } else {
          pick = lowest_bits(run_starts(avail, c), take - acc);
        }
        if (pick) {
          const uint64_t mask = expand_runs(pick, c);
          const uint64_t old = ptx::atom_and_acquire(bits + w, ~mask);
          const uint64_t gotbits = old & mask;
          got = run_starts(gotbits, c) & pick;
          // a run with a slice still on its way back (a free from the block's
          // previous life, see pin_block) is not taken: return what of it
          // this fetch-and cleared
          const uint64_t partial = gotbits & ~expand_runs(got, c);
          if (partial) ptx::red_or_relaxed(bits + w, partial);
          avail = old & ~mask;
        } else {
          avail = 0;
        }
        whole = false;
        if (run_starts(avail, c) == 0) {
          w = (w + 1) & 63;
          avail = ~0ull;
          whole = true;
        }
      }
      got = ptx::shfl64(grp, got, leader);
      gw = __shfl_sync(grp, gw, leader);
      const uint32_t kk = (uint32_t)__popcll(got);
      if (g_rank >= acc && g_rank < acc + kk) my_slice = (int)(gw * 64 + (uint32_t)ptx::nth_set_bit(got, (int)(g_rank - acc)));
      acc += kk;
    }
    if (acc < take && lane == (uint32_t)leader) {
      release_live(st, b, (take - acc) * c);
      count(st, GAL_CTR_CLAIM_SHORT);
    }
    if (my_slice >= 0) {
      result = block_address(st, b, t) + ((uint64_t)my_slice << (st->min_shift + (int)t));
      done = true;
    }
    if (refill && lane == (uint32_t)leader) {
      count(st, GAL_CTR_REPLACE_REFILL);
      uint32_t nb;
      replace_slot(st, slot, (uint64_t)b, t, r, ADOPT_ROOMY, &nb);  // no nearly-full blocks
    }
  }
  if (result == nullptr) count(st, GAL_CTR_OOM_SLICE);
  return result;
}

// Warp-aggregated slice free: one fetch-or per (block, word) and one
// release of the live count per block.
__device__ inline void free_slice(const gal_state_t *st, uint64_t seg, uint32_t t, uint64_t off_s,
                                  uint32_t width = 32) {
  const uint32_t active = __activemask() & tile_mask(width);
  const int bis = block_index_shift(st);
  const uint64_t i = off_s >> (st->block_shift_min + (int)t);
  const uint64_t b = (seg << bis) + i;
  const uint32_t slice = (uint32_t)(off_s >> (st->min_shift + (int)t)) & (GAL_BLOCK_SLICES - 1);
  const uint32_t word = slice >> 6;
  const uint32_t bit = slice & 63;
  // a block of the largest tree serves one run length, kept in its meta word
  // (stable while this allocation holds the block out of its segment, and
  // written before the pointer reached this thread: a plain load suffices)
  uint32_t c = 1;
  if (t == (uint32_t)st->num_trees - 1) c = 1u << meta_run(st->block_meta[b]);
  const uint64_t mask = ((c >= 64) ? ~0ull : ((1ull << c) - 1)) << bit;
  const uint32_t lane = ptx::laneid();

  const uint32_t wpeers = __match_any_sync(active, (unsigned long long)((b << 6) | word));
  const uint64_t or_mask = ptx::reduce_or64(wpeers, mask);
  const uint32_t bpeers = __match_any_sync(active, (unsigned long long)b);
  const uint32_t total = __reduce_add_sync(bpeers, c);
  // one fence orders every lane's payload writes before both returns: the
  // next owner of these slices (through the bitmap) and the block's retire
  // (through the live count) see them; the two returns need no order between
  // them (see pin_block)
  __syncwarp(active);
  ptx::fence_acq_rel();
  if (lane == (uint32_t)(__ffs((int)wpeers) - 1)) ptx::red_or_relaxed(st->block_bits + (b << 6) + word, or_mask);
  if (lane == (uint32_t)(__ffs((int)bpeers) - 1)) release_live(st, b, total, true);
}

// ---- block and segment tiers ---------------------------------------------

__device__ inline GAL_COLD void *malloc_block(const gal_state_t *st, uint32_t bt, uint64_t tid) {
  bool adopted = false;
  const uint32_t b = request_block(st, bt, 0, 1, tid, ADOPT_NONE, &adopted);
  if (b == GAL_EMPTY_BLOCK) {
    count(st, GAL_CTR_OOM_BLOCK);
    return nullptr;
  }
  own_block(st, b, bt, 0, GAL_STATE_WHOLE, 1);
  return block_address(st, b, bt);
}

__device__ inline GAL_COLD void *malloc_segment(const gal_state_t *st, uint64_t nseg) {
  const uint64_t max_n = 0xFFFEull - (uint64_t)st->num_trees - 1;
  if (nseg > st->num_segments || nseg > max_n) {
    count(st, GAL_CTR_OOM_SEGMENT);
    return nullptr;
  }
  // the reference spins on this lock without bound (gallatin.cuh:796)
  uint32_t spins = 0;
  while (!try_lock(st, kSegmentLockBit)) {
    if (++spins >= st->lock_spins) {
      count(st, GAL_CTR_TIMEOUT);
      return nullptr;
    }
    backoff((int)(spins < 4096 ? spins : 4096));
  }
  const uint64_t first = veb::gather_run(&st->segment_tree, nseg);
  unlock(st, kSegmentLockBit);
  if (first == veb::kFail) {
    count(st, GAL_CTR_OOM_SEGMENT);
    return nullptr;
  }
  const unsigned short tag = (unsigned short)((uint64_t)st->num_trees + 1 + nseg);
  if (atomicCAS((unsigned short *)(st->chunk_ids + first), (unsigned short)GAL_FREE_SEGMENT, tag) !=
      (unsigned short)GAL_FREE_SEGMENT) {
    count(st, GAL_CTR_CORRUPT);
    return nullptr;
  }
  return st->memory + (first << st->segment_shift);
}

__device__ inline GAL_COLD void free_segment(const gal_state_t *st, uint64_t seg, uint16_t id) {
  const uint64_t n = (uint64_t)id - (uint64_t)st->num_trees - 1;
  if (atomicCAS((unsigned short *)(st->chunk_ids + seg), (unsigned short)id, (unsigned short)GAL_FREE_SEGMENT) !=
      (unsigned short)id) {
    count(st, GAL_CTR_BAD_FREE);
    return;
  }
  __threadfence();
  veb::return_run(&st->segment_tree, seg, n);
  clear_nomem(st);
}

// ---- zeroing for GAL_FLAG_CALLOC ------------------------------------------

// Zero [p, p + bytes) for every lane of `active` with bytes != 0; the lanes
// of `active` store 16 B each per step, one lane's range at a time, so a full
// warp writes 512 contiguous bytes per step. bytes is a multiple of 16 and p
// 16-byte aligned (every allocation is). Ends with the lanes' stores ordered
// before anything each lane does next (__syncwarp orders memory among the
// lanes it joins, so one lane's later release fence covers them all).
__device__ inline void zero_ranges(uint32_t active, char *p, uint64_t bytes) {
  const uint32_t lane = ptx::laneid();
  const uint32_t rank = (uint32_t)__popc(active & ((1u << lane) - 1u));
  const uint32_t group = (uint32_t)__popc(active);
  uint32_t pending = __ballot_sync(active, bytes != 0);
  while (pending) {
    const int src = __ffs((int)pending) - 1;
    pending &= pending - 1;
    uint4 *q = (uint4 *)__shfl_sync(active, (unsigned long long)p, src);
    const uint64_t n16 = __shfl_sync(active, (unsigned long long)bytes, src) >> 4;
    for (uint64_t i = rank; i < n16; i += group) q[i] = make_uint4(0u, 0u, 0u, 0u);
  }
  __syncwarp(active);
}

// Bytes a live allocation at arena offset `off` spans, read from the
// metadata that free uses (0 for a pointer free would reject): the slice run
// of its block, a whole block-tier block, or its segments. The span never
// reaches past the end of the block (slice and block tiers) or of the arena
// (segment tier) that holds `off`, so even a pointer that was freed twice,
// whose block words may no longer describe it, cannot make the zeroing
// write outside the arena.
__device__ inline uint64_t allocation_span(const gal_state_t *st, uint64_t off) {
  if (off >= st->arena_bytes) return 0;
  const uint64_t seg = off >> st->segment_shift;
  const uint16_t id = st->chunk_ids[seg];
  if (id < (uint16_t)st->num_trees) {
    const uint32_t t = id;
    const int block_shift = st->block_shift_min + (int)t;
    const uint64_t b = (seg << block_index_shift(st)) + ((off & (st->segment_bytes - 1)) >> block_shift);
    // state (WHOLE or not) and run length cannot change while the allocation
    // is live; read past L1 all the same
    const uint64_t m = ptx::ld_relaxed(st->block_meta + b);
    const int slice_shift = st->min_shift + (int)t;
    const uint64_t room = (1ull << block_shift) - (off & ((1ull << block_shift) - 1));
    uint64_t span = (uint64_t)GAL_BLOCK_SLICES << slice_shift;
    if (meta_state(m) != GAL_STATE_WHOLE)
      span = ((t == (uint32_t)st->num_trees - 1) ? (1ull << meta_run(m)) : 1ull) << slice_shift;
    return span < room ? span : room;
  }
  if (id != GAL_FREE_SEGMENT && id > (uint16_t)st->num_trees) {
    const uint64_t span = ((uint64_t)id - (uint64_t)st->num_trees - 1) << st->segment_shift;
    return span < st->arena_bytes - off ? span : st->arena_bytes - off;
  }
  return 0;
}

// ---- dropping freed bytes from L2 ----------------------------------------
//
// A freed allocation's bytes are dead, but the lines its owner wrote sit
// dirty in L2 and are written back to HBM when evicted: for allocations that
// live briefly (written, read, freed) that write-back is most of their HBM
// traffic. free drops those lines instead (discard.global.L2), for single
// slices of 128 B to 4 KiB: their lines are whole, aligned and owned by this
// allocation alone (smaller slices share lines with their neighbours; larger
// spans cost more discards than the write-back they save when, as for pages,
// most of the span is never written). The discards come before the free's
// fence, so the next owner, who acquires the slice after the free's release,
// writes after them.
constexpr int kDiscardMaxShift = 12;  // largest slice whose lines are dropped: 4 KiB

// Bytes at arena offset `off` whose lines free may drop, or 0.
__device__ __forceinline__ uint64_t discard_span(const gal_state_t *st, uint64_t off) {
  if (off >= st->arena_bytes) return 0;
  const uint64_t seg = off >> st->segment_shift;
  const uint16_t id = st->chunk_ids[seg];
  if (id >= (uint16_t)st->num_trees) return 0;
  const int slice_shift = st->min_shift + (int)id;
  if (slice_shift < 7 || slice_shift > kDiscardMaxShift) return 0;
  if (id == (uint16_t)st->num_trees - 1) {
    // a block of the largest tree serves runs of one length: drop only single slices
    const int block_shift = st->block_shift_min + (int)id;
    const uint64_t b = (seg << block_index_shift(st)) + ((off & (st->segment_bytes - 1)) >> block_shift);
    if (meta_run(st->block_meta[b]) != 0) return 0;
  }
  return 1ull << slice_shift;
}

// Drop the lines of [p, p + bytes) for every lane of `active` with bytes != 0
// (bytes a multiple of 128, p 128-byte aligned): the lanes issue one discard
// per line, one lane's range at a time, 4 KiB per full-warp step.
__device__ inline void discard_ranges(uint32_t active, char *p, uint64_t bytes) {
  const uint32_t lane = ptx::laneid();
  const uint32_t rank = (uint32_t)__popc(active & ((1u << lane) - 1u));
  const uint32_t group = (uint32_t)__popc(active);
  uint32_t pending = __ballot_sync(active, bytes != 0);
  while (pending) {
    const int src = __ffs((int)pending) - 1;
    pending &= pending - 1;
    char *q = (char *)__shfl_sync(active, (unsigned long long)p, src);
    const uint64_t lines = __shfl_sync(active, (unsigned long long)bytes, src) >> 7;
    for (uint64_t i = rank; i < lines; i += group) ptx::discard_l2(q + (i << 7));
  }
}

// ---- public entry points -------------------------------------------------

// `width` limits warp aggregation to tiles of 8, 16 or 32 lanes (the
// reference groups the whole coalesced warp, gallatin.cuh:883-885).
__device__ __forceinline__ void *malloc(const gal_state_t *st, uint64_t size, uint32_t width = 32) {
  const size_class sc = classify(st, size);
  if (sc.tier == TIER_SLICE) return malloc_slice(st, sc.tree, (uint32_t)(__ffs((int)sc.count) - 1), width);
  if (sc.tier == TIER_BLOCK) return malloc_block(st, sc.tree, veb::thread_tid());
  return malloc_segment(st, sc.nseg);
}

__device__ inline void free(const gal_state_t *st, void *ptr, uint32_t width = 32) {
  // calloc mode: the freeing lanes zero their allocations together before
  // any of them hands its bytes back (st->flags is the same for every lane)
  if (st->flags & GAL_FLAG_CALLOC)
    zero_ranges(__activemask(), (char *)ptr,
                ptr == nullptr ? 0 : allocation_span(st, (uint64_t)((char *)ptr - st->memory)));
  else if ((st->flags & (GAL_FLAG_HOST_ARENA | GAL_FLAG_DROP_FREED)) == GAL_FLAG_DROP_FREED)
    discard_ranges(__activemask(), (char *)ptr,
                   ptr == nullptr ? 0 : discard_span(st, (uint64_t)((char *)ptr - st->memory)));
  if (ptr == nullptr) return;
  const uint64_t off = (uint64_t)((char *)ptr - st->memory);
  if (off >= st->arena_bytes) {
    count(st, GAL_CTR_BAD_FREE);
    return;
  }
  const uint64_t seg = off >> st->segment_shift;
  // the segment's tag cannot change while the allocation is live, and it was
  // set before the pointer was handed out, so a plain (L1-cacheable) load
  // sees it (freeing a pointer twice is undefined, as in the reference)
  const uint16_t id = st->chunk_ids[seg];
  if (id < (uint16_t)st->num_trees) {
    free_slice(st, seg, id, off & (st->segment_bytes - 1), width);
  } else if (id != GAL_FREE_SEGMENT && id > (uint16_t)st->num_trees) {
    free_segment(st, seg, id);
  } else {
    count(st, GAL_CTR_BAD_FREE);
  }
}

// malloc, except that a slice request of a class whose last slot
// replacement found no block (and no block or segment has gone back to a
// pool since) returns NULL at once: for callers with somewhere else to go,
// such as the device-first / host-arena pair, which would otherwise pay for
// a search that is known to fail.
__device__ __forceinline__ void *malloc_unless_full(const gal_state_t *st, uint64_t size, uint32_t width = 32) {
  const size_class sc = classify(st, size);
  if (sc.tier == TIER_SLICE) {
    const uint32_t k = sc.tree + (uint32_t)(__ffs((int)sc.count) - 1);
    if ((ptx::ld_relaxed(st->nomem) >> k) & 1u) return nullptr;
  }
  return malloc(st, size, width);
}

// Bytes a request of `size` really occupies (reference get_allocated_size,
// gallatin.cuh:1152-1183, whose tier test compares against num_trees the
// same way).
__device__ inline uint64_t allocated_size(const gal_state_t *st, uint64_t size) {
  if (size < 16) size = 16;
  const int bit_size = ceil_log2(size);
  const int tree = (size < (1ull << st->min_shift)) ? 0 : bit_size - st->min_shift;
  if (tree > st->num_trees) {
    const int block_tree = bit_size - st->block_shift_min;
    if (block_tree > st->num_trees) return (((size - 1) >> st->segment_shift) + 1) << st->segment_shift;
  }
  return 1ull << bit_size;
}

__device__ __forceinline__ bool owns_allocation(const gal_state_t *st, const void *ptr) {
  return (uint64_t)((const char *)ptr - st->memory) < st->arena_bytes;
}

// Detach the block a slot holds (maintenance; no mallocs may run).
__device__ inline void flush_slot(const gal_state_t *st, uint64_t *slot) {
  const uint64_t sv = ptx::ld_relaxed(slot);
  const uint32_t b = (uint32_t)sv;
  if (b == GAL_EMPTY_BLOCK || (sv & GAL_SLOT_REPLACING)) return;
  if (atomicCAS((unsigned long long *)slot, sv, (unsigned long long)GAL_EMPTY_BLOCK) != sv) return;
  detach_block(st, b);
}

}  // namespace gal

#endif  // GALLATIN_GB300_ALLOC_CUH

// Device van Emde Boas style 64-ary bit trie over segment ids.
//
// Semantics follow the reference veb_tree (veb.cuh:528-1228) operation by
// operation so that ordered, single-threaded query sets give bit-identical
// results and bit-identical layer state:
//   * layer count ceil(bitlen(U)/6), layer 0 on top (veb.cuh:544-561)
//   * remove floats up while the touched word had popcount 1 (veb.cuh:737-755)
//   * insert floats up while the old word had popcount 30 (veb.cuh:757-773)
//   * insert_force_update floats up while the old word was empty (:775-798)
//   * successor is strict (> x) and does one float-up/float-down pass
//     (:836-873); successor_thorough repeats it (:878-916)
//   * lock_offset, find_first_valid_index, find_random_valid_index, malloc,
//     malloc_first (:918-1032), with the MurmurHash64A double-hash start.
//
// What differs, and why:
//   * layers live inline in gal_veb_t (no layers[i]->bits pointer chase) and
//     every word access is a gpu-scope relaxed load or atomic;
//   * remove re-checks the child word after clearing a parent bit and puts
//     the bit back if the child was refilled meanwhile, so a concurrent
//     insert can never leave a non-empty word invisible to successor search
//     (in sequential use the re-check never fires);
//   * successor_thorough has an iteration cap (the reference loop is
//     unbounded) and reports the cap through the allocator's counters;
//   * gather_run / return_run replace gather_multiple / return_multiple
//     (veb.cuh:323-523,1160-1218): the search first walks the reference's
//     order (top word down, runs that touch bit 0 of a word >= 1) and then
//     falls back to an exhaustive search, so it only fails when no run of n
//     free bits exists; upper layers are kept equal to the OR of their
//     children.
#ifndef GALLATIN_GB300_VEB_CUH
#define GALLATIN_GB300_VEB_CUH

#include <stdint.h>

#include "ptx.cuh"
#include "murmur.cuh"
#include "state.h"

namespace gal {
namespace veb {

constexpr uint64_t kFail = ~0ull;
constexpr int kMaxAttempts = 15;      // VEB_MAX_ATTEMPTS (veb.cuh:59)
constexpr int kRestartCutoff = 30;    // VEB_RESTART_CUTOFF (veb.cuh:56)
constexpr int kThoroughLimit = 1 << 12;  // bounds every retry loop below

__device__ __forceinline__ uint64_t *word_ptr(const gal_veb_t *t, int layer, uint64_t high) {
  return t->bits[layer] + high;
}

__device__ __forceinline__ int find_next(const gal_veb_t *t, int layer, uint64_t high, int low) {
  if (high >= t->layer_universe[layer]) return -1;
  uint64_t w = ptx::ld_relaxed(word_ptr(t, layer, high));
  if (low < 0) return __ffsll((long long)w) - 1;
  if (low >= 63) return -1;
  return __ffsll((long long)(w & (~0ull << (low + 1)))) - 1;
}

__device__ __forceinline__ bool float_up(int &layer, uint64_t &high, int &low) {
  layer -= 1;
  low = (int)(high & 63);
  high >>= 6;
  return layer >= 0;
}

__device__ __forceinline__ bool float_down(const gal_veb_t *t, int &layer, uint64_t &high, int &low) {
  layer += 1;
  high = (high << 6) + (uint64_t)low;
  low = -1;
  return layer < t->num_layers;
}

__device__ __forceinline__ bool query(const gal_veb_t *t, uint64_t x) {
  uint64_t w = ptx::ld_relaxed(word_ptr(t, t->num_layers - 1, x >> 6));
  return (w >> (x & 63)) & 1ull;
}

// The word at `layer`/`high` just became empty: clear its bit in the parent
// and keep floating up while the parent word had popcount 1 before the
// clear (the reference's rule, veb.cuh:748). When this thread's clear is
// what emptied the child, the child is re-read after the parent bit is
// cleared; if a concurrent insert refilled it, the parent bit goes back and
// the float stops. Sequentially the re-read always sees the empty child, so
// results and layer state match the reference even on trees whose upper
// layers plain insert() left stale.
__device__ __forceinline__ void float_up_clear(const gal_veb_t *t, int layer, uint64_t high) {
  int low = 0;
  bool child_emptied = true;
  while (true) {
    const int child_layer = layer;
    const uint64_t child_high = high;
    if (!float_up(layer, high, low)) break;
    const uint64_t bit = 1ull << low;
    const uint64_t old = ptx::atom_and_relaxed(word_ptr(t, layer, high), ~bit);
    if (child_emptied && ptx::ld_relaxed(word_ptr(t, child_layer, child_high)) != 0) {
      ptx::atom_or_relaxed(word_ptr(t, layer, high), bit);
      break;
    }
    if (__popcll(old) != 1) break;
    child_emptied = (old & ~bit) == 0;
  }
}

// Set the parent bits above a word at `layer`/`high` that was empty before
// an insert (`old` is the pre-insert word).
__device__ __forceinline__ void float_up_set(const gal_veb_t *t, int layer, uint64_t high, uint64_t old) {
  int low = 0;
  while (__popcll(old) == 0 && float_up(layer, high, low)) {
    old = ptx::atom_or_relaxed(word_ptr(t, layer, high), 1ull << low);
  }
}

__device__ __forceinline__ bool remove(const gal_veb_t *t, uint64_t x) {
  const int leaf = t->num_layers - 1;
  const uint64_t high = x >> 6;
  const uint64_t bit = 1ull << (x & 63);
  uint64_t old = ptx::atom_and_relaxed(word_ptr(t, leaf, high), ~bit);
  if (!(old & bit)) return false;
  if (__popcll(old) == 1) float_up_clear(t, leaf, high);
  return true;
}

__device__ __forceinline__ bool insert(const gal_veb_t *t, uint64_t x) {
  int layer = t->num_layers - 1;
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  uint64_t old = ptx::atom_or_relaxed(word_ptr(t, layer, high), 1ull << low);
  if (old & (1ull << low)) return false;
  while (__popcll(old) == kRestartCutoff && float_up(layer, high, low)) {
    old = ptx::atom_or_relaxed(word_ptr(t, layer, high), 1ull << low);
  }
  return true;
}

__device__ __forceinline__ bool insert_force_update(const gal_veb_t *t, uint64_t x) {
  const int leaf = t->num_layers - 1;
  const uint64_t high = x >> 6;
  const uint64_t bit = 1ull << (x & 63);
  uint64_t old = ptx::atom_or_relaxed(word_ptr(t, leaf, high), bit);
  if (old & bit) return false;
  float_up_set(t, leaf, high, old);
  return true;
}

__device__ __forceinline__ uint64_t successor(const gal_veb_t *t, uint64_t x) {
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  int layer = t->num_layers - 1;
  while (true) {
    if (find_next(t, layer, high, low) == -1) {
      if (layer == 0) return kFail;
      float_up(layer, high, low);
      continue;
    }
    break;
  }
  while (layer != t->num_layers - 1) {
    low = find_next(t, layer, high, low);
    if (low == -1) return kFail;
    float_down(t, layer, high, low);
  }
  low = find_next(t, layer, high, low);
  if (low == -1) return kFail;
  return (high << 6) + (uint64_t)low;
}

// `capped` is set when the iteration cap ends the search (never in
// sequential use of a consistent tree).
__device__ __forceinline__ uint64_t successor_thorough(const gal_veb_t *t, uint64_t x, bool *capped = nullptr) {
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  int layer = t->num_layers - 1;
  for (int iter = 0; iter < kThoroughLimit; ++iter) {
    while (true) {
      if (find_next(t, layer, high, low) == -1) {
        if (layer == 0) return kFail;
        float_up(layer, high, low);
        continue;
      }
      break;
    }
    while (layer != t->num_layers - 1) {
      low = find_next(t, layer, high, low);
      if (low == -1) break;
      float_down(t, layer, high, low);
    }
    low = find_next(t, layer, high, low);
    if (low != -1) return (high << 6) + (uint64_t)low;
  }
  if (capped) *capped = true;
  return kFail;
}

__device__ __forceinline__ uint64_t lock_offset(const gal_veb_t *t, uint64_t start) {
  if (query(t, start) && remove(t, start)) return start;
  for (int iter = 0; iter < kThoroughLimit; ++iter) {
    start = successor_thorough(t, start);
    if (start == kFail) return start;
    if (remove(t, start)) return start;
  }
  return kFail;
}

__device__ __forceinline__ uint64_t find_first_valid_index(const gal_veb_t *t) {
  if (query(t, 0)) return 0;
  return successor_thorough(t, 0);
}

// The reference derives tid from threadIdx/blockIdx inside the call
// (veb.cuh:948); here it is an argument so batch kernels and the op runner
// can pass it explicitly. thread_tid() gives the reference's value.
__device__ __forceinline__ uint64_t thread_tid() {
  return (uint64_t)(threadIdx.x + blockIdx.x * blockDim.x);
}

__device__ __forceinline__ uint64_t find_random_valid_index(const gal_veb_t *t, uint64_t tid) {
  const uint64_t hash1 = murmur64a_u64(tid, t->seed);
  const uint64_t hash2 = murmur64a_u64(tid, hash1);
  for (int attempts = 0; attempts < kMaxAttempts; ++attempts) {
    uint64_t start = (hash1 + (uint64_t)attempts * hash2) % t->universe;
    if (query(t, start)) return start;
    uint64_t index = successor_thorough(t, start);
    if (index != kFail) return index;
  }
  return successor_thorough(t, 0);
}

__device__ __forceinline__ uint64_t malloc_first(const gal_veb_t *t) {
  for (int attempts = 0; attempts < kMaxAttempts; ++attempts) {
    uint64_t offset = lock_offset(t, 0);
    if (offset != kFail) return offset;
  }
  return kFail;
}

__device__ __forceinline__ uint64_t malloc_random(const gal_veb_t *t, uint64_t tid) {
  const uint64_t hash1 = murmur64a_u64(tid, t->seed);
  const uint64_t hash2 = murmur64a_u64(tid, hash1);
  for (int attempts = 0; attempts < kMaxAttempts; ++attempts) {
    uint64_t start = (hash1 + (uint64_t)attempts * hash2) % t->universe;
    uint64_t offset = lock_offset(t, start);
    if (offset != kFail) return offset;
  }
  return lock_offset(t, 0);
}

// ---- searches of the allocator's own trees ------------------------------
//
// The allocator maintains its trees with insert_force_update and remove
// only, so every upper-layer bit is the OR of its child word (up to the
// moment of a concurrent change). On such a tree the smallest set id >= x is
// one well-defined answer, and these searches reach it in fewer dependent
// loads than query + successor_thorough: the query and the first leaf scan
// share one load, which reads the aligned pair of leaf words holding x
// (layers are allocated with an even number of words), so a successor in the
// next word needs no float up; upper layers are visited only past the pair.
// The op-for-op reference semantics above stay the parity surface.

// Smallest set id >= x, or kFail. A word found empty on the way down (a
// concurrent remove) resumes the search after it; the loop is bounded.
__device__ inline uint64_t find_at_or_after(const gal_veb_t *t, uint64_t x) {
  if (x >= t->universe) return kFail;
  const int leaf = t->num_layers - 1;
  const uint64_t w = x >> 6;
  uint64_t p0, p1;
  ptx::ld_relaxed_v2(word_ptr(t, leaf, w & ~1ull), p0, p1);
  const uint64_t cur = ((w & 1) ? p1 : p0) & (~0ull << (x & 63));
  if (cur) return (w << 6) + (uint64_t)(__ffsll((long long)cur) - 1);
  if (!(w & 1) && p1) return ((w + 1) << 6) + (uint64_t)(__ffsll((long long)p1) - 1);
  // search after word `idx` of `layer`
  int layer = leaf;
  uint64_t idx = w | 1;
  for (int iter = 0; iter < kThoroughLimit; ++iter) {
    // float up to the first layer whose word holds a set bit after idx's
    while (true) {
      if (layer == 0) return kFail;
      const uint64_t pw = idx >> 6;
      const int pb = (int)(idx & 63);
      const uint64_t v = pb == 63 ? 0ull : (ptx::ld_relaxed(word_ptr(t, layer - 1, pw)) & (~0ull << (pb + 1)));
      layer -= 1;
      if (v) {
        idx = (pw << 6) + (uint64_t)(__ffsll((long long)v) - 1);
        layer += 1;  // idx is now a word of the child layer
        break;
      }
      idx = pw;
    }
    // float down along first set bits
    while (true) {
      const uint64_t v = ptx::ld_relaxed(word_ptr(t, layer, idx));
      if (v == 0) break;  // emptied meanwhile: search after it
      const uint64_t b = (uint64_t)(__ffsll((long long)v) - 1);
      if (layer == leaf) return (idx << 6) + b;
      idx = (idx << 6) + b;
      layer += 1;
    }
  }
  return kFail;
}

// Claim the smallest set id (remove it), or kFail when none is set.
__device__ inline uint64_t claim_first(const gal_veb_t *t) {
  for (int iter = 0; iter < kThoroughLimit; ++iter) {
    const uint64_t x = find_at_or_after(t, 0);
    if (x == kFail) return kFail;
    if (remove(t, x)) return x;
  }
  return kFail;
}

// A set id from a hashed start (MurmurHash64A of tid under the tree's seed,
// as find_random_valid_index starts), wrapping to the smallest set id.
__device__ inline uint64_t find_hashed(const gal_veb_t *t, uint64_t tid) {
  const uint64_t start = murmur64a_u64(tid, t->seed) % t->universe;
  const uint64_t x = find_at_or_after(t, start);
  return (x != kFail || start == 0) ? x : find_at_or_after(t, 0);
}

// ---- contiguous runs (segment tier) -------------------------------------

__device__ __forceinline__ uint64_t run_mask(int lo, int len) {
  return (len >= 64) ? ~0ull : (((1ull << len) - 1) << lo);
}

// Try to claim leaf bits [start, start+n). On any bit already taken, give
// back what was claimed and return false. Words that become empty clear
// their parent bits.
__device__ inline bool claim_run(const gal_veb_t *t, uint64_t start, uint64_t n) {
  const int leaf = t->num_layers - 1;
  uint64_t pos = start;
  uint64_t left = n;
  while (left > 0) {
    const uint64_t w = pos >> 6;
    const int lo = (int)(pos & 63);
    const int len = (int)((left < (uint64_t)(64 - lo)) ? left : (uint64_t)(64 - lo));
    const uint64_t mask = run_mask(lo, len);
    uint64_t old = ptx::atom_and_acquire(word_ptr(t, leaf, w), ~mask);
    if ((old & mask) != mask) {
      // roll back this word's bits we did get, then the earlier words
      uint64_t got = old & mask;
      if (got) ptx::atom_or_relaxed(word_ptr(t, leaf, w), got);
      uint64_t p = start;
      while (p < pos) {
        const uint64_t pw = p >> 6;
        const int plo = (int)(p & 63);
        const uint64_t rem = pos - p;
        const int plen = (int)((rem < (uint64_t)(64 - plo)) ? rem : (uint64_t)(64 - plo));
        uint64_t pold = ptx::atom_or_relaxed(word_ptr(t, leaf, pw), run_mask(plo, plen));
        float_up_set(t, leaf, pw, pold);
        p += (uint64_t)plen;
      }
      return false;
    }
    if ((old & ~mask) == 0) float_up_clear(t, leaf, w);
    pos += (uint64_t)len;
    left -= (uint64_t)len;
  }
  return true;
}

// Number of consecutive free bits going down from bit p (inclusive).
__device__ __forceinline__ uint64_t free_run_down(const gal_veb_t *t, int64_t p, uint64_t cap) {
  const int leaf = t->num_layers - 1;
  uint64_t count = 0;
  while (p >= 0 && count < cap) {
    const uint64_t w = (uint64_t)p >> 6;
    const int b = (int)(p & 63);
    uint64_t word = ptx::ld_relaxed(word_ptr(t, leaf, w));
    // bits 0..b of the word, shifted so bit b is the top bit
    uint64_t below = word << (63 - b);
    // count leading ones of `below`
    int ones = __clzll((long long)~below);
    if (ones > b + 1) ones = b + 1;
    count += (uint64_t)ones;
    if (ones < b + 1) break;
    p -= ones;
  }
  return count;
}

// Contiguous run of n free ids. Returns the first id or kFail.
// The caller serialises gatherers (allocator segment-tier lock).
__device__ inline uint64_t gather_run(const gal_veb_t *t, uint64_t n) {
  if (n == 0 || n > t->universe) return kFail;
  const int leaf = t->num_layers - 1;
  const uint64_t words = t->layer_words[leaf];
  for (int pass = 0; pass < 64; ++pass) {
    bool raced = false;
    // phase 1: the reference order
    for (uint64_t w = words - 1; w >= 1 && !raced; --w) {
      uint64_t word = ptx::ld_relaxed(word_ptr(t, leaf, w));
      int c = (~word == 0) ? 64 : (__ffsll((long long)~word) - 1);
      if (c == 0) continue;
      uint64_t end = (w << 6) + (uint64_t)c;  // exclusive
      uint64_t have = (uint64_t)c;
      if (have < n) have += free_run_down(t, (int64_t)(w << 6) - 1, n - have);
      if (have < n) continue;
      if (claim_run(t, end - n, n)) return end - n;
      raced = true;
    }
    if (raced) continue;
    // phase 2: exhaustive, highest run end first
    int64_t p = (int64_t)(t->universe) - 1;
    while (p >= (int64_t)n - 1) {
      uint64_t word = ptx::ld_relaxed(word_ptr(t, leaf, (uint64_t)p >> 6));
      if (!((word >> (p & 63)) & 1ull)) {
        // skip the used bits below p within this word
        const int b = (int)(p & 63);
        uint64_t below = (b == 63) ? word : (word & ((1ull << (b + 1)) - 1));
        if (below == 0) {
          p = (int64_t)(((uint64_t)p >> 6) << 6) - 1;
        } else {
          p = (int64_t)(((uint64_t)p >> 6) << 6) + (63 - __clzll((long long)below));
        }
        continue;
      }
      uint64_t have = free_run_down(t, p, n);
      if (have >= n) {
        uint64_t start = (uint64_t)p + 1 - n;
        if (claim_run(t, start, n)) return start;
        raced = true;
        break;
      }
      p -= (int64_t)have;
    }
    if (!raced) return kFail;
  }
  return kFail;
}

// Give back ids [start, start+n); words that were empty set their parents.
__device__ inline void return_run(const gal_veb_t *t, uint64_t start, uint64_t n) {
  const int leaf = t->num_layers - 1;
  uint64_t pos = start;
  uint64_t left = n;
  while (left > 0) {
    const uint64_t w = pos >> 6;
    const int lo = (int)(pos & 63);
    const int len = (int)((left < (uint64_t)(64 - lo)) ? left : (uint64_t)(64 - lo));
    uint64_t old = ptx::atom_or_relaxed(word_ptr(t, leaf, w), run_mask(lo, len));
    float_up_set(t, leaf, w, old);
    pos += (uint64_t)len;
    left -= (uint64_t)len;
  }
}

}  // namespace veb
}  // namespace gal

#endif  // GALLATIN_GB300_VEB_CUH

/*
 * ORACLE — test infrastructure only. Nothing in the product links this file;
 * only tests/, the smoke check and bench.py's CPU-baseline leg may load it.
 *
 * Single-threaded CPU restatement of the reference vEB tree
 * (saltsystemslab/gallatin include/gallatin/allocators/veb.cuh) used to
 * check the GPU implementation bit for bit on ordered query sets.
 *
 * Two modes share every single-bit operation and differ only in the
 * contiguous-run operations:
 *   mode 0 "reference as written": layer::gather_multiple (veb.cuh:323-452)
 *          with its top-down scan that never starts in word 0 and its final
 *          rollback(0, ...) (veb.cuh:447), veb_tree::gather_multiple
 *          (veb.cuh:1160-1196, maybe_remove_layer_bits :1100-1126) and
 *          return_multiple (veb.cuh:1198-1218, maybe_return_layer_bits
 *          :1128-1154, which sets a parent bit only when the child word is
 *          full). The quirk counter records when a call hits one of the two
 *          behaviours that leave the tree inconsistent (a final rollback that
 *          sets bits in word 0, or a return that leaves a non-empty child
 *          under a clear parent bit).
 *   mode 1 "GB300": gather_run / return_run of include/gallatin_gb300/veb.cuh
 *          (reference scan order first, then an exhaustive search; upper
 *          layers kept equal to the OR of their children).
 *
 * Parity of this oracle is pinned by tests/golden/veb_golden.npz, produced by
 * running the reference's own veb_tree on a GB300 (tests/golden/gen_veb_golden.py).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MAXL 8
#define FAIL (~0ull)
#define VEB_MAX_ATTEMPTS 15   /* veb.cuh:59 */
#define VEB_RESTART_CUTOFF 30 /* veb.cuh:56 */
#define THOROUGH_LIMIT (1 << 20)

typedef struct {
  uint64_t seed, universe;
  int L;
  uint64_t *bits[MAXL];
  uint64_t luniv[MAXL], lwords[MAXL];
  int mode;
  uint64_t quirks;
} veb;

typedef struct {
  uint32_t code, tid;
  uint64_t arg, arg2;
} veb_op;

static inline int popc(uint64_t x) { return __builtin_popcountll(x); }
static inline int ffs64(uint64_t x) { return x ? __builtin_ctzll(x) + 1 : 0; }
static inline uint64_t bitmask(uint64_t n) { return n >= 64 ? ~0ull : ((1ull << n) - 1); }

/* MurmurHash64A, 8-byte key (murmurhash.cuh:20-61) */
static uint64_t murmur64a_u64(uint64_t key, uint64_t seed) {
  const uint64_t m = 0xc6a4a7935bd1e995ull;
  const int r = 47;
  uint64_t h = seed ^ (8ull * m);
  uint64_t k = key * m;
  k ^= k >> r;
  k *= m;
  h ^= k;
  h *= m;
  h ^= h >> r;
  h *= m;
  h ^= h >> r;
  return h;
}

static int veb_init(veb *t, uint64_t universe, uint64_t seed, int mode) {
  memset(t, 0, sizeof(*t));
  if (universe == 0) return -1;
  int max_height = 64 - __builtin_clzll(universe);
  int L = (max_height - 1) / 6 + 1; /* veb.cuh:544-548 */
  if (L > MAXL) return -1;
  t->seed = seed;
  t->universe = universe;
  t->L = L;
  t->mode = mode;
  uint64_t u = universe;
  for (int i = 0; i < L; i++) {
    int layer = L - 1 - i;
    uint64_t words = (u - 1) / 64 + 1;
    t->luniv[layer] = u;
    t->lwords[layer] = words;
    t->bits[layer] = (uint64_t *)calloc(words, 8);
    if (!t->bits[layer]) return -1;
    for (uint64_t w = 0; w < words; w++) { /* init_bits: ids < u set (veb.cuh:72-84) */
      uint64_t left = u - w * 64;
      t->bits[layer][w] = left >= 64 ? ~0ull : ((1ull << left) - 1);
    }
    u = (u - 1) / 64 + 1;
  }
  return 0;
}

static void veb_free(veb *t) {
  for (int i = 0; i < t->L; i++) free(t->bits[i]);
}

static int find_next(veb *t, int layer, uint64_t high, int low) { /* veb.cuh:250-275 */
  if (high >= t->luniv[layer]) return -1;
  uint64_t w = t->bits[layer][high];
  if (low == -1) return ffs64(w) - 1;
  return ffs64(w & ~bitmask((uint64_t)low + 1)) - 1;
}

static int float_up(int *layer, uint64_t *high, int *low) { /* veb.cuh:697-704 */
  *layer -= 1;
  *low = (int)(*high & 63);
  *high >>= 6;
  return *layer >= 0;
}

static int float_down(veb *t, int *layer, uint64_t *high, int *low) { /* veb.cuh:706-712 */
  *layer += 1;
  *high = (*high << 6) + (uint64_t)*low;
  *low = -1;
  return *layer < t->L;
}

static uint64_t raw_and(uint64_t *w, uint64_t v) { uint64_t o = *w; *w &= v; return o; }
static uint64_t raw_or(uint64_t *w, uint64_t v) { uint64_t o = *w; *w |= v; return o; }

static int veb_remove(veb *t, uint64_t x) { /* veb.cuh:737-755 */
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  int layer = t->L - 1;
  uint64_t old = raw_and(&t->bits[layer][high], ~(1ull << low));
  if (!(old & (1ull << low))) return 0;
  while (popc(old) == 1 && float_up(&layer, &high, &low)) old = raw_and(&t->bits[layer][high], ~(1ull << low));
  return 1;
}

static int veb_insert(veb *t, uint64_t x) { /* veb.cuh:757-773 */
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  int layer = t->L - 1;
  uint64_t old = raw_or(&t->bits[layer][high], 1ull << low);
  if (old & (1ull << low)) return 0;
  while (popc(old) == VEB_RESTART_CUTOFF && float_up(&layer, &high, &low))
    old = raw_or(&t->bits[layer][high], 1ull << low);
  return 1;
}

static int veb_insert_force(veb *t, uint64_t x) { /* veb.cuh:775-798 */
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  int layer = t->L - 1;
  uint64_t old = raw_or(&t->bits[layer][high], 1ull << low);
  if (old & (1ull << low)) return 0;
  while (popc(old) == 0 && float_up(&layer, &high, &low)) old = raw_or(&t->bits[layer][high], 1ull << low);
  return 1;
}

static int veb_query(veb *t, uint64_t x) { /* veb.cuh:824-829 */
  return (int)((t->bits[t->L - 1][x >> 6] >> (x & 63)) & 1ull);
}

static uint64_t veb_successor(veb *t, uint64_t x) { /* veb.cuh:836-873 */
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  int layer = t->L - 1;
  while (1) {
    if (find_next(t, layer, high, low) == -1) {
      if (layer == 0) return FAIL;
      float_up(&layer, &high, &low);
      continue;
    }
    break;
  }
  while (layer != t->L - 1) {
    low = find_next(t, layer, high, low);
    if (low == -1) return FAIL;
    float_down(t, &layer, &high, &low);
  }
  low = find_next(t, layer, high, low);
  if (low == -1) return FAIL;
  return (high << 6) + (uint64_t)low;
}

static uint64_t veb_successor_thorough(veb *t, uint64_t x) { /* veb.cuh:878-916 */
  uint64_t high = x >> 6;
  int low = (int)(x & 63);
  int layer = t->L - 1;
  for (int iter = 0; iter < THOROUGH_LIMIT; iter++) {
    while (1) {
      if (find_next(t, layer, high, low) == -1) {
        if (layer == 0) return FAIL;
        float_up(&layer, &high, &low);
        continue;
      }
      break;
    }
    while (layer != t->L - 1) {
      low = find_next(t, layer, high, low);
      if (low == -1) break;
      float_down(t, &layer, &high, &low);
    }
    low = find_next(t, layer, high, low);
    if (low != -1) return (high << 6) + (uint64_t)low;
  }
  return FAIL - 1; /* iteration cap: never reached on the golden sets */
}

static uint64_t veb_lock_offset(veb *t, uint64_t start) { /* veb.cuh:918-937 */
  if (veb_query(t, start) && veb_remove(t, start)) return start;
  for (int iter = 0; iter < THOROUGH_LIMIT; iter++) {
    start = veb_successor_thorough(t, start);
    if (start == FAIL || start == FAIL - 1) return start;
    if (veb_remove(t, start)) return start;
  }
  return FAIL - 1;
}

static uint64_t veb_find_first(veb *t) { /* veb.cuh:940-944 */
  if (veb_query(t, 0)) return 0;
  return veb_successor_thorough(t, 0);
}

static uint64_t veb_find_random(veb *t, uint64_t tid) { /* veb.cuh:946-977 */
  uint64_t hash1 = murmur64a_u64(tid, t->seed);
  uint64_t hash2 = murmur64a_u64(tid, hash1);
  for (int attempts = 0; attempts < VEB_MAX_ATTEMPTS; attempts++) {
    uint64_t start = (hash1 + (uint64_t)attempts * hash2) % t->universe;
    if (veb_query(t, start)) return start;
    uint64_t index = veb_successor_thorough(t, start);
    if (index != FAIL) return index;
  }
  return veb_successor_thorough(t, 0);
}

static uint64_t veb_malloc_first(veb *t) { /* veb.cuh:979-991 */
  for (int attempts = 0; attempts < VEB_MAX_ATTEMPTS; attempts++) {
    uint64_t offset = veb_lock_offset(t, 0);
    if (offset != FAIL) return offset;
  }
  return FAIL;
}

static uint64_t veb_malloc(veb *t, uint64_t tid) { /* veb.cuh:993-1032 */
  uint64_t hash1 = murmur64a_u64(tid, t->seed);
  uint64_t hash2 = murmur64a_u64(tid, hash1);
  for (int attempts = 0; attempts < VEB_MAX_ATTEMPTS; attempts++) {
    uint64_t start = (hash1 + (uint64_t)attempts * hash2) % t->universe;
    uint64_t offset = veb_lock_offset(t, start);
    if (offset != FAIL) return offset;
  }
  return veb_lock_offset(t, 0);
}

/* ---- mode 0: the reference's run operations as written ---------------- */

static int cfcll(uint64_t bits) { /* alloc_utils.cuh:440-453 */
  int p = popc(bits);
  if (p == 0 || p == 64) return p;
  return ffs64(~bits) - 1;
}

/* returns 0 if the write would be out of bounds */
static int layer_rollback(veb *t, int layer, uint64_t start_block, uint64_t bits_to_set) { /* veb.cuh:305-321 */
  uint64_t *bits = t->bits[layer];
  while (bits_to_set > 64) {
    if (start_block >= t->lwords[layer]) return 0;
    bits[start_block] |= ~0ull;
    bits_to_set -= 64;
    start_block++;
  }
  if (start_block >= t->lwords[layer]) return bits_to_set == 0;
  bits[start_block] |= bitmask(bits_to_set);
  return 1;
}

#define OOB_ERROR (FAIL - 2)

static uint64_t layer_gather_ref(veb *t, uint64_t num_contiguous) { /* veb.cuh:323-452 */
  int layer = t->L - 1;
  uint64_t *bits = t->bits[layer];
  uint64_t start_block = t->lwords[layer] - 1;
  uint64_t num_needed = num_contiguous;
  int guard = 0;
  while (start_block != 0) {
    if (++guard > 1 << 20) return OOB_ERROR;
    num_contiguous = num_needed;
    int contig_start = cfcll(bits[start_block]);
    if (contig_start == 0) {
      start_block -= 1;
      continue;
    }
    if ((uint64_t)contig_start >= num_contiguous) {
      uint64_t acq = bitmask(num_contiguous) << (contig_start - num_contiguous);
      uint64_t acquired = raw_and(&bits[start_block], ~acq);
      if ((uint64_t)popc(acquired & acq) == num_contiguous) return start_block * 64 + (contig_start - num_contiguous);
      raw_or(&bits[start_block], acq & acquired);
      continue;
    }
    uint64_t acquired = raw_and(&bits[start_block], ~bitmask(contig_start));
    int succeeded = 1;
    if (popc(acquired & bitmask(contig_start)) == contig_start) {
      num_contiguous -= contig_start;
      while (num_contiguous > 64) {
        if (start_block == 0) return OOB_ERROR; /* reference would index bits[-1] */
        start_block--;
        acquired = raw_and(&bits[start_block], 0ull);
        if (popc(acquired) != 64) {
          raw_or(&bits[start_block], acquired);
          if (!layer_rollback(t, layer, start_block + 1, num_needed - num_contiguous)) return OOB_ERROR;
          succeeded = 0;
          break;
        }
        num_contiguous -= 64;
      }
      if (!succeeded) continue;
      if (start_block == 0) return OOB_ERROR;
      start_block--;
      uint64_t final_mask = bitmask(num_contiguous) << (64 - num_contiguous);
      uint64_t final_bits = raw_and(&bits[start_block], ~final_mask);
      if ((uint64_t)popc(final_bits & final_mask) == num_contiguous) return start_block * 64 + 64 - num_contiguous;
      raw_or(&bits[start_block], final_mask & final_bits);
      if (!layer_rollback(t, layer, start_block + 1, num_needed - num_contiguous)) return OOB_ERROR;
      continue;
    } else {
      raw_or(&bits[start_block], acquired & bitmask(contig_start));
      continue;
    }
  }
  if (num_needed - num_contiguous > 0) t->quirks++; /* rollback(0, >0) sets bits in word 0 */
  if (!layer_rollback(t, layer, 0, num_needed - num_contiguous)) return OOB_ERROR;
  return FAIL;
}

static uint64_t free_run_down(veb *t, int64_t p, uint64_t cap);

/* true when some run of n free leaf bits exists */
static int has_run(veb *t, uint64_t n) {
  int64_t p = (int64_t)t->universe - 1;
  while (p >= (int64_t)n - 1) {
    uint64_t have = free_run_down(t, p, n);
    if (have >= n) return 1;
    p -= (int64_t)(have ? have : 1);
  }
  return 0;
}

static uint64_t gather_ref(veb *t, uint64_t n) { /* veb.cuh:1160-1196 */
  uint64_t found = layer_gather_ref(t, n);
  if (found == FAIL && has_run(t, n)) t->quirks++; /* the scan missed a run that exists */
  if (found == FAIL || found == OOB_ERROR) return found;
  uint64_t original = found;
  uint64_t num = n;
  for (int i = t->L - 2; i >= 0; i--) {
    uint64_t tread_high = (found + num - 1) / 64 + 1;
    uint64_t tread_low = found / 64;
    found = tread_low;
    num = tread_high - tread_low;
    for (uint64_t wb = found; wb < found + num; wb++) { /* maybe_remove_layer_bits */
      if (t->bits[i + 1][wb] == 0) t->bits[i][wb / 64] &= ~(1ull << (wb % 64));
    }
  }
  return original;
}

static void layer_return_range(veb *t, int layer, uint64_t start, uint64_t num) { /* veb.cuh:495-523 */
  uint64_t block_index = start / 64;
  int block_start = (int)(start % 64);
  while (num + (uint64_t)block_start > 64) {
    int added = 64 - block_start;
    t->bits[layer][block_index] |= bitmask(added) << block_start;
    block_start = 0;
    block_index += 1;
    num -= (uint64_t)added;
  }
  t->bits[layer][block_index] |= bitmask(num) << block_start;
}

static void return_ref(veb *t, uint64_t start, uint64_t num) { /* veb.cuh:1198-1218 */
  layer_return_range(t, t->L - 1, start, num);
  for (int i = t->L - 2; i >= 0; i--) {
    uint64_t tread_high = (start + num - 1) / 64 + 1;
    uint64_t tread_low = start / 64;
    start = tread_low;
    num = tread_high - tread_low;
    for (uint64_t wb = start; wb < start + num; wb++) { /* maybe_return_layer_bits */
      uint64_t child = t->bits[i + 1][wb];
      if (popc(child) == 64) {
        t->bits[i][wb / 64] |= 1ull << (wb % 64);
      } else if (child != 0 && !((t->bits[i][wb / 64] >> (wb % 64)) & 1ull)) {
        t->quirks++; /* non-empty child left under a clear parent bit */
      }
    }
  }
}

/* ---- mode 1: GB300 run operations (include/gallatin_gb300/veb.cuh) ----- */

static void float_up_clear(veb *t, int layer, uint64_t high) {
  int low = 0;
  while (1) {
    if (!float_up(&layer, &high, &low)) break;
    uint64_t old = raw_and(&t->bits[layer][high], ~(1ull << low));
    if (popc(old) != 1) break;
  }
}

static void float_up_set(veb *t, int layer, uint64_t high, uint64_t old) {
  int low = 0;
  while (popc(old) == 0 && float_up(&layer, &high, &low)) old = raw_or(&t->bits[layer][high], 1ull << low);
}

static uint64_t free_run_down(veb *t, int64_t p, uint64_t cap) {
  int leaf = t->L - 1;
  uint64_t count = 0;
  while (p >= 0 && count < cap) {
    uint64_t w = t->bits[leaf][(uint64_t)p >> 6];
    int b = (int)(p & 63);
    int ones = 0;
    while (ones <= b && ((w >> (b - ones)) & 1ull)) ones++;
    count += (uint64_t)ones;
    if (ones < b + 1) break;
    p -= ones;
  }
  return count;
}

static void claim_run(veb *t, uint64_t start, uint64_t n) {
  int leaf = t->L - 1;
  uint64_t pos = start, left = n;
  while (left > 0) {
    uint64_t w = pos >> 6;
    int lo = (int)(pos & 63);
    uint64_t len = left < (uint64_t)(64 - lo) ? left : (uint64_t)(64 - lo);
    uint64_t mask = (len >= 64) ? ~0ull : (((1ull << len) - 1) << lo);
    uint64_t old = raw_and(&t->bits[leaf][w], ~mask);
    if ((old & ~mask) == 0) float_up_clear(t, leaf, w);
    pos += len;
    left -= len;
  }
}

static uint64_t gather_run(veb *t, uint64_t n) {
  if (n == 0 || n > t->universe) return FAIL;
  int leaf = t->L - 1;
  uint64_t words = t->lwords[leaf];
  for (uint64_t w = words - 1; w >= 1; w--) { /* phase 1: the reference order */
    uint64_t word = t->bits[leaf][w];
    int c = (~word == 0) ? 64 : ffs64(~word) - 1;
    if (c == 0) continue;
    uint64_t end = (w << 6) + (uint64_t)c;
    uint64_t have = (uint64_t)c;
    if (have < n) have += free_run_down(t, (int64_t)(w << 6) - 1, n - have);
    if (have < n) continue;
    claim_run(t, end - n, n);
    return end - n;
  }
  int64_t p = (int64_t)t->universe - 1; /* phase 2: exhaustive, highest run end first */
  while (p >= (int64_t)n - 1) {
    uint64_t word = t->bits[leaf][(uint64_t)p >> 6];
    if (!((word >> (p & 63)) & 1ull)) {
      p--;
      continue;
    }
    uint64_t have = free_run_down(t, p, n);
    if (have >= n) {
      uint64_t start = (uint64_t)p + 1 - n;
      claim_run(t, start, n);
      return start;
    }
    p -= (int64_t)have;
  }
  return FAIL;
}

static void return_run(veb *t, uint64_t start, uint64_t n) {
  int leaf = t->L - 1;
  uint64_t pos = start, left = n;
  while (left > 0) {
    uint64_t w = pos >> 6;
    int lo = (int)(pos & 63);
    uint64_t len = left < (uint64_t)(64 - lo) ? left : (uint64_t)(64 - lo);
    uint64_t mask = (len >= 64) ? ~0ull : (((1ull << len) - 1) << lo);
    uint64_t old = raw_or(&t->bits[leaf][w], mask);
    float_up_set(t, leaf, w, old);
    pos += len;
    left -= len;
  }
}

/* ---- op runner ---------------------------------------------------------- */

static uint64_t run_op(veb *t, const veb_op *op) {
  switch (op->code) {
    case 0: return (uint64_t)veb_insert(t, op->arg);
    case 1: return (uint64_t)veb_insert_force(t, op->arg);
    case 2: return (uint64_t)veb_remove(t, op->arg);
    case 3: return (uint64_t)veb_query(t, op->arg);
    case 4: return veb_successor(t, op->arg);
    case 5: return veb_successor_thorough(t, op->arg);
    case 6: return veb_lock_offset(t, op->arg);
    case 7: return veb_malloc_first(t);
    case 8: return veb_find_first(t);
    case 9: return veb_find_random(t, op->tid);
    case 10: return veb_malloc(t, op->tid);
    case 11: return t->mode == 0 ? gather_ref(t, op->arg) : gather_run(t, op->arg);
    case 12:
      if (t->mode == 0) return_ref(t, op->arg, op->arg2);
      else return_run(t, op->arg, op->arg2);
      return 0;
    case 13: {
      uint64_t fill = 0;
      for (uint64_t w = 0; w < t->lwords[t->L - 1]; w++) fill += (uint64_t)popc(t->bits[t->L - 1][w]);
      return fill;
    }
    default: return FAIL - 1;
  }
}

/* Number of layers and words per layer (top first) of a tree over universe. */
int oracle_veb_shape(uint64_t universe, uint64_t *words_out /* MAXL */) {
  if (universe == 0) return -1;
  int max_height = 64 - __builtin_clzll(universe);
  int L = (max_height - 1) / 6 + 1;
  uint64_t u = universe;
  for (int i = 0; i < L; i++) {
    words_out[L - 1 - i] = (u - 1) / 64 + 1;
    u = (u - 1) / 64 + 1;
  }
  return L;
}

/* Run `n` ops on a full tree; write per-op results, the final layers
 * (concatenated, top first) and, per op, the quirk count so far.
 * Returns the total quirk count, or -1 on a bad argument. */
int64_t oracle_veb_run(uint64_t universe, uint64_t seed, int mode, const veb_op *ops, uint64_t n, uint64_t *results,
                       uint64_t *layers_out, uint64_t *quirks_out) {
  veb t;
  if (veb_init(&t, universe, seed, mode) != 0) return -1;
  for (uint64_t i = 0; i < n; i++) {
    results[i] = run_op(&t, &ops[i]);
    if (quirks_out) quirks_out[i] = t.quirks;
  }
  if (layers_out) {
    uint64_t off = 0;
    for (int l = 0; l < t.L; l++) {
      memcpy(layers_out + off, t.bits[l], t.lwords[l] * 8);
      off += t.lwords[l];
    }
  }
  int64_t q = (int64_t)t.quirks;
  veb_free(&t);
  return q;
}

uint64_t oracle_murmur64a_u64(uint64_t key, uint64_t seed) { return murmur64a_u64(key, seed); }

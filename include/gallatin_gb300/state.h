/*
 * Device-resident state of one GB300 Gallatin allocator instance.
 *
 * This layout is shared by the C-ABI host library (which builds it) and by
 * the header-only device code that user kernels inline (which reads it).
 * Everything here is plain C so that host code without nvcc can see it.
 *
 * HBM layout (all arrays are separate cudaMalloc allocations, 256-B aligned):
 *   memory          arena, num_segments * segment_bytes (with
 *                   GAL_FLAG_HOST_ARENA: pinned, mapped host memory the GPU
 *                   reaches over the C2C link; the metadata stays in HBM)
 *   chunk_ids       u16[num_segments]   0xFFFF = unformatted, t < num_trees =
 *                   formatted for slice tree t, num_trees+1+n = head of an
 *                   n-segment allocation (reference memory_table.cuh:823-851,
 *                   gallatin.cuh:802)
 *   seg_avail       i32[num_segments]   free blocks left in a formatted
 *                   segment; GAL_SEG_GATE when the segment is unformatted
 *   seg_block_bits  u64[num_segments * seg_block_words]  1 = block free
 *   block_meta      u64[num_segments * blocks_per_segment]  see GAL_META_*
 *   block_bits      u64[num_segments * blocks_per_segment * 64]  1 = slice free
 *   slots           u64[total_slots]    pinned block per (slot class, SM slot)
 *   veb bit layers  one u64 array per layer per tree: the segment tree and
 *                   the per-tree sub trees over segment ids, and per slot
 *                   class two trees over block ids (detached blocks with room,
 *                   and the subset that drained to half a block or less)
 *
 * Slot classes: class t < num_trees-1 serves single slices of tree t; the
 * largest tree has one class per run length 2^r (r = 0 .. num_classes -
 * num_trees), class num_trees-1+r. A block of the largest tree serves one
 * run length for as long as it is out of its segment, so its free slices
 * always form aligned runs of that length.
 */
#ifndef GALLATIN_GB300_STATE_H
#define GALLATIN_GB300_STATE_H

#include <stdint.h>

#define GAL_BLOCK_SLICES 4096u
#define GAL_BLOCK_WORDS 64u
#define GAL_MAX_TREES 24
#define GAL_MAX_LAYERS 8
#define GAL_FREE_SEGMENT 0xFFFFu
#define GAL_EMPTY_BLOCK 0xFFFFFFFFu
/* seg_avail of an unformatted segment: far below any reachable count, so
 * stale decrements and their undos never make it look formatted. */
#define GAL_SEG_GATE (-(1 << 28))

/* block_meta word:
 *   bits  0-31  live: slices reserved or held (reservations precede claims)
 *   bits 32-39  tree id the block is formatted for
 *   bits 40-41  state: FREE (in its segment's pool), PINNED (serving a slot),
 *               DETACHED (no longer pinned; recycled when live reaches 0),
 *               WHOLE (one block-tier allocation)
 *   bits 42-45  log2 of the run length the block serves (largest tree only)
 *   bit  46     reused: pinned again while it still held slices, so its free
 *               slices are scattered and the cursor does not point at them
 *   bit  47     fresh: pinned from its segment with every bitmap bit set and
 *               the cursor at 0; while the cursor has not passed 4096 the
 *               reserved positions are exactly the free slices
 *   bits 48-63  cursor: position hint for the next claim, wraps mod 2^16
 * All transitions are atomic adds of field deltas (or a CAS for the
 * conditional retire) so concurrent reservations and their undos commute. */
#define GAL_META_LIVE_MASK 0xFFFFFFFFull
#define GAL_META_TREE_SHIFT 32
#define GAL_META_STATE_SHIFT 40
#define GAL_META_RUN_SHIFT 42
#define GAL_META_REUSED_BIT (1ull << 46)
#define GAL_META_FRESH_BIT (1ull << 47)
#define GAL_META_CURSOR_SHIFT 48
#define GAL_STATE_FREE 0u
#define GAL_STATE_PINNED 1u
#define GAL_STATE_DETACHED 2u
#define GAL_STATE_WHOLE 3u
/* a detached block is listed for early reuse once live <= this */
#define GAL_ROOMY_MARK (GAL_BLOCK_SLICES / 2)

/* gal_state_t.flags */
#define GAL_FLAG_HOST_ARENA 1u /* arena in pinned host memory (reference host_only, memory_table.cuh:521-540) */
#define GAL_FLAG_CALLOC 2u     /* arena zeroed at creation and every free zeroes its bytes before they
                                  can be handed out again, so malloc returns zeroed memory (reference
                                  running_calloc, gallatin.cuh:1306-1369) */
#define GAL_FLAG_DROP_FREED 4u /* a free of one slice of 128 B to 4 KiB on an HBM arena (without
                                  GAL_FLAG_CALLOC) drops the slice's lines from L2 without writing them
                                  back: the bytes are dead, so HBM never sees them. Off by default: it
                                  saves HBM writes but costs L2 requests (see gal::discard_ranges). */

/* default bound on the segment-tier lock wait: 2^20 tries with a backoff of
 * up to ~1 us each, about a second */
#define GAL_DEFAULT_LOCK_SPINS (1u << 20)

/* slot word: low 32 bits block id (GAL_EMPTY_BLOCK when none), bit 32 set
 * while one leader is replacing the block. */
#define GAL_SLOT_REPLACING (1ull << 32)

/* diagnostic counters (device, u64 each) */
enum gal_counter_id {
  GAL_CTR_OOM_SLICE = 0,
  GAL_CTR_OOM_BLOCK = 1,
  GAL_CTR_OOM_SEGMENT = 2,
  GAL_CTR_TIMEOUT = 3,
  GAL_CTR_BAD_FREE = 4,
  GAL_CTR_CORRUPT = 5,
  GAL_CTR_BLOCK_PINS = 6,
  GAL_CTR_SEGMENT_ATTACH = 7,
  GAL_CTR_SEGMENT_RETIRE = 8,
  GAL_CTR_BLOCK_RETIRE = 9,
  GAL_CTR_REPLACE_EMPTY = 10, /* slot had no block yet */
  GAL_CTR_REPLACE_FULL = 11,  /* pinned block had no room left */
  GAL_CTR_REPLACE_FRAG = 12,  /* unused: blocks serve one run length, so runs do not fragment */
  GAL_CTR_CLAIM_SHORT = 13,   /* reservation held but bits not found in time */
  GAL_CTR_STALE_SLOT = 14,    /* slot changed between read and reservation */
  GAL_CTR_SLOT_BUSY = 15,     /* slot was being replaced */
  GAL_CTR_REPLACE_REFILL = 16, /* pinned block replaced ahead of filling up */
  GAL_CTR_ADOPT = 17,          /* detached block with room pinned again (arena full) */
  GAL_CTR_ADOPT_ROOMY = 18,    /* detached block at or under half live pinned again */
  GAL_CTR_NOMEM = 19,          /* slot found full with no block to replace it */
  GAL_CTR_TREE_PINS = 32,     /* + tree id: blocks pinned per tree */
  GAL_NUM_COUNTERS = 64
};

typedef struct gal_veb_t {
  uint64_t seed;
  uint64_t universe;
  int32_t num_layers;
  int32_t pad_;
  uint64_t *bits[GAL_MAX_LAYERS];          /* layer 0 = top, num_layers-1 = leaf */
  uint64_t layer_universe[GAL_MAX_LAYERS]; /* items in each layer */
  uint64_t layer_words[GAL_MAX_LAYERS];    /* u64 words in each layer */
} gal_veb_t;

typedef struct gal_state_t {
  /* geometry: every size is a power of two */
  uint64_t segment_bytes;
  uint64_t num_segments;
  uint64_t arena_bytes;
  int32_t segment_shift;    /* log2(segment_bytes) */
  int32_t min_shift;        /* log2(smallest slice) */
  int32_t max_shift;        /* log2(largest slice) */
  int32_t num_trees;        /* max_shift - min_shift + 1 */
  int32_t block_shift_min;  /* log2(smallest slice * 4096) */
  uint32_t blocks_per_segment;     /* for tree 0; tree t has this >> t */
  uint32_t seg_block_words;        /* u64 words per segment block bitmap */
  uint32_t num_classes;            /* slot classes, see above */
  uint32_t num_sms;
  uint32_t total_slots;
  uint32_t flags;                  /* GAL_FLAG_* */
  uint32_t lock_spins;             /* tries of the segment-tier lock before a
                                      segment-tier malloc gives up (NULL and
                                      GAL_CTR_TIMEOUT); GAL_DEFAULT_LOCK_SPINS */
  uint32_t slot_count[GAL_MAX_TREES];
  uint32_t slot_offset[GAL_MAX_TREES];
  uint64_t seed;

  char *memory;
  uint16_t *chunk_ids;
  int32_t *seg_avail;
  uint64_t *seg_block_bits;
  uint64_t *block_meta;
  uint64_t *block_bits;
  uint64_t *slots;
  uint32_t *locks;                 /* bit t: tree t attach lock; bit 31: segment tier */
  uint32_t *nomem;                 /* bit k: the last replacement for slot class k found no
                                      block (a hint; cleared by the next one that does) */
  unsigned long long *counters;    /* GAL_NUM_COUNTERS */

  gal_veb_t segment_tree;
  gal_veb_t sub_trees[GAL_MAX_TREES];
  /* per slot class: DETACHED blocks (universe = all block ids) that a slot
   * can pin again when no fresh block is left, so their free slices stay
   * reachable; roomy_trees lists those with live <= GAL_ROOMY_MARK, which
   * are pinned again before a fresh block is taken */
  gal_veb_t adopt_trees[GAL_MAX_TREES];
  gal_veb_t roomy_trees[GAL_MAX_TREES];
} gal_state_t;

#endif /* GALLATIN_GB300_STATE_H */

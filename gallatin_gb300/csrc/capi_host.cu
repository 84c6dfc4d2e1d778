// C ABI: allocator lifetime, geometry, stats and metadata dumps.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cstddef>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "capi_internal.h"

namespace {

std::mutex g_registry_mutex;
std::unordered_map<const void *, gal_allocator *> g_registry;
char g_last_error[512] = "";

bool is_pow2(uint64_t v) { return v != 0 && (v & (v - 1)) == 0; }
int log2_exact(uint64_t v) { return 63 - __builtin_clzll(v); }

template <class T>
int device_alloc(gal_allocator *h, T **out, uint64_t count, const char *what) {
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T) > 0 ? count * sizeof(T) : 16);
  if (e != cudaSuccess) {
    galcapi::fail_cuda(e, what);
    return GAL_ERR_NOMEM;
  }
  h->device_allocs.push_back(p);
  *out = (T *)p;
  return GAL_OK;
}

void free_all(std::vector<void *> &allocs) {
  for (void *p : allocs) cudaFree(p);
  allocs.clear();
}

}  // namespace

namespace galcapi {

void set_error(const char *msg) {
  snprintf(g_last_error, sizeof(g_last_error), "%s", msg);
}

int fail_cuda(cudaError_t e, const char *what) {
  snprintf(g_last_error, sizeof(g_last_error), "%s: %s", what, cudaGetErrorString(e));
  return (e == cudaErrorMemoryAllocation) ? GAL_ERR_NOMEM : GAL_ERR_CUDA;
}

int fail_invalid(const char *what) {
  set_error(what);
  return GAL_ERR_INVALID;
}

int build_veb(gal_veb_t *t, uint64_t universe, uint64_t seed, bool full, std::vector<void *> &allocs) {
  if (universe == 0) return fail_invalid("vEB universe must be positive");
  memset(t, 0, sizeof(*t));
  const int max_height = 64 - __builtin_clzll(universe);
  const int layers = (max_height - 1) / 6 + 1;  // reference veb.cuh:544-548
  if (layers > GAL_MAX_LAYERS) return fail_invalid("vEB universe too large");
  t->seed = seed;
  t->universe = universe;
  t->num_layers = layers;
  uint64_t u = universe;
  for (int i = 0; i < layers; ++i) {
    const int layer = layers - 1 - i;
    const uint64_t words = (u - 1) / 64 + 1;
    t->layer_universe[layer] = u;
    t->layer_words[layer] = words;
    // an even number of words, the last one zero when words is odd, so the
    // allocator's searches can read any aligned pair of words in one 128-bit
    // load (no bit is ever set past the layer's universe)
    const uint64_t padded = (words + 1) & ~1ull;
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, padded * sizeof(uint64_t));
    if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc vEB layer");
    allocs.push_back(p);
    t->bits[layer] = (uint64_t *)p;
    std::vector<uint64_t> host(padded, 0);
    if (full) {
      for (uint64_t w = 0; w < words; ++w) {
        const uint64_t lo = w * 64;
        const uint64_t left = u - lo;
        host[w] = left >= 64 ? ~0ull : ((1ull << left) - 1);
      }
    }
    e = cudaMemcpy(p, host.data(), padded * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemcpy vEB layer");
    u = (u - 1) / 64 + 1;
  }
  return GAL_OK;
}

}  // namespace galcapi

using galcapi::fail_invalid;

extern "C" const char *gal_last_error(void) { return g_last_error; }

extern "C" int gal_create(uint64_t max_bytes, uint64_t seed, uint64_t segment_bytes, uint64_t min_size,
                          uint64_t max_size, uint32_t min_slots, gal_allocator **out) {
  return gal_create_ex(max_bytes, seed, segment_bytes, min_size, max_size, min_slots, 0, out);
}

extern "C" int gal_create_ex(uint64_t max_bytes, uint64_t seed, uint64_t segment_bytes, uint64_t min_size,
                             uint64_t max_size, uint32_t min_slots, uint32_t flags, gal_allocator **out) {
  if (out == nullptr) return fail_invalid("out is NULL");
  *out = nullptr;
  if (flags & ~(GAL_FLAG_HOST_ARENA | GAL_FLAG_CALLOC | GAL_FLAG_DROP_FREED)) return fail_invalid("unknown flags");
  if (!is_pow2(segment_bytes) || !is_pow2(min_size) || !is_pow2(max_size))
    return fail_invalid("segment, min and max sizes must be powers of two");
  if (max_size < min_size) return fail_invalid("max_size < min_size");
  if (segment_bytes < max_size * 4096) return fail_invalid("segment_bytes must be >= max_size * 4096");
  if (max_size < 32 * min_size) return fail_invalid("max_size must be >= 32 * min_size");
  const uint64_t num_segments = max_bytes / segment_bytes;  // reference alloc_utils.cuh:224
  if (num_segments == 0) return fail_invalid("max_bytes smaller than one segment");
  const int min_shift = log2_exact(min_size);
  const int max_shift = log2_exact(max_size);
  const int num_trees = max_shift - min_shift + 1;
  if (num_trees > GAL_MAX_TREES) return fail_invalid("too many size classes");
  if (num_segments * (segment_bytes / (min_size * 4096)) >= 0xFFFFFFF0ull)
    return fail_invalid("too many blocks: block ids are 32-bit");
  if ((uint64_t)num_trees + 2 + 1 > 0xFFFEull) return fail_invalid("too many size classes");

  int dev = 0;
  cudaDeviceProp prop;
  GAL_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  GAL_CUDA_TRY(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");

  gal_allocator *h = new gal_allocator();
  h->d_state = nullptr;
  h->d_classes = nullptr;
  h->d_classes_bytes = 0;
  h->d_stats = nullptr;
  h->d_breqs = h->d_boffs = h->d_btable = nullptr;
  h->d_breqs_bytes = h->d_boffs_bytes = h->d_btable_bytes = 0;
  h->copy_stream = nullptr;
  h->copy_event = nullptr;
  h->d_bsorted = nullptr;
  h->d_bbins = nullptr;
  h->d_bsorted_bytes = h->d_bbins_bytes = 0;
  h->d_serve = nullptr;
  h->d_serve_bytes = 0;
  h->d_ftable = nullptr;
  h->d_ftable_bytes = 0;
  h->host_arena = nullptr;
  h->d_fused = nullptr;
  h->min_size = min_size;
  h->max_size = max_size;
  gal_state_t &s = h->hs;
  memset(&s, 0, sizeof(s));
  s.segment_bytes = segment_bytes;
  s.num_segments = num_segments;
  s.arena_bytes = num_segments * segment_bytes;
  s.segment_shift = log2_exact(segment_bytes);
  s.min_shift = min_shift;
  s.max_shift = max_shift;
  s.num_trees = num_trees;
  s.block_shift_min = min_shift + 12;
  s.blocks_per_segment = (uint32_t)(segment_bytes >> s.block_shift_min);
  // even, so a segment's free-block words start 16-byte aligned and can be
  // read in pairs (a word past blocks_per_segment stays zero)
  s.seg_block_words = ((s.blocks_per_segment + 63) / 64 + 1) & ~1u;
  // the largest tree serves runs of 1, 2, 4 ... slices up to half the
  // smallest block (min_size << 11 bytes), one slot class per run length
  const int max_run = 12 - num_trees > 0 ? 12 - num_trees : 0;
  s.num_classes = (uint32_t)(num_trees + max_run);
  s.num_sms = (uint32_t)prop.multiProcessorCount;
  s.seed = seed;
  s.flags = flags;
  s.lock_spins = GAL_DEFAULT_LOCK_SPINS;
  // Pinned blocks per slot class: one per SM for small trees; for large
  // trees as many as a quarter of the arena split evenly over the trees
  // affords (a block of tree t is 4096 slices of min << t bytes). A run
  // class of 2^r slices of the largest tree gets that tree's count >> (r - 1)
  // (at least 2): longer runs are asked for more rarely. Slots are filled on first use, so a
  // class that is never asked for pins nothing.
  if (min_slots == 0) min_slots = 4;
  const uint64_t budget = s.arena_bytes / (4ull * (uint64_t)num_trees);
  uint32_t total = 0;
  for (uint32_t k = 0; k < s.num_classes; ++k) {
    const int t = (int)k < num_trees ? (int)k : num_trees - 1;
    const uint64_t block_bytes = 4096ull * (min_size << t);
    uint64_t c = budget / block_bytes;
    if (c > s.num_sms) c = s.num_sms;
    if (c < min_slots) c = min_slots;
    if ((int)k > num_trees) c = (c >> (k - (uint32_t)num_trees)) > 2 ? (c >> (k - (uint32_t)num_trees)) : 2;
    s.slot_count[k] = (uint32_t)c;
    s.slot_offset[k] = total;
    total += (uint32_t)c;
  }
  s.total_slots = total;

  const uint64_t nblocks = num_segments * s.blocks_per_segment;
  int rc = GAL_OK;
  auto cleanup = [&](int code) {
    free_all(h->device_allocs);
    if (h->host_arena) cudaFreeHost(h->host_arena);
    delete h;
    return code;
  };
  if (flags & GAL_FLAG_HOST_ARENA) {
    // pinned host pages mapped into the GPU's address space (the reference's
    // host_only table, memory_table.cuh:521-540); with unified addressing the
    // device address equals the host address
    if (!prop.canMapHostMemory) return cleanup(fail_invalid("device cannot map host memory"));
    cudaError_t e = cudaHostAlloc((void **)&h->host_arena, s.arena_bytes, cudaHostAllocMapped);
    if (e != cudaSuccess) {
      h->host_arena = nullptr;
      return cleanup(galcapi::fail_cuda(e, "cudaHostAlloc arena"));
    }
    e = cudaHostGetDevicePointer((void **)&s.memory, h->host_arena, 0);
    if (e != cudaSuccess) return cleanup(galcapi::fail_cuda(e, "cudaHostGetDevicePointer arena"));
    if (flags & GAL_FLAG_CALLOC) memset(h->host_arena, 0, s.arena_bytes);
  } else {
    if ((rc = device_alloc(h, &s.memory, s.arena_bytes, "cudaMalloc arena")) != GAL_OK) return cleanup(rc);
    if (flags & GAL_FLAG_CALLOC) {
      const cudaError_t e = cudaMemset(s.memory, 0, s.arena_bytes);
      if (e != cudaSuccess) return cleanup(galcapi::fail_cuda(e, "memset arena"));
    }
  }
  if ((rc = device_alloc(h, &s.chunk_ids, num_segments, "cudaMalloc chunk_ids")) != GAL_OK) return cleanup(rc);
  if ((rc = device_alloc(h, &s.seg_avail, num_segments, "cudaMalloc seg_avail")) != GAL_OK) return cleanup(rc);
  if ((rc = device_alloc(h, &s.seg_block_bits, num_segments * s.seg_block_words, "cudaMalloc seg bits")) != GAL_OK)
    return cleanup(rc);
  if ((rc = device_alloc(h, &s.block_meta, nblocks, "cudaMalloc block_meta")) != GAL_OK) return cleanup(rc);
  if ((rc = device_alloc(h, &s.block_bits, nblocks * 64, "cudaMalloc block_bits")) != GAL_OK) return cleanup(rc);
  if ((rc = device_alloc(h, &s.slots, total, "cudaMalloc slots")) != GAL_OK) return cleanup(rc);
  if ((rc = device_alloc(h, &s.locks, 1, "cudaMalloc locks")) != GAL_OK) return cleanup(rc);
  if ((rc = device_alloc(h, &s.nomem, 1, "cudaMalloc nomem")) != GAL_OK) return cleanup(rc);
  if ((rc = device_alloc(h, &s.counters, GAL_NUM_COUNTERS, "cudaMalloc counters")) != GAL_OK) return cleanup(rc);
  if ((rc = device_alloc(h, &h->d_stats, 8, "cudaMalloc stats")) != GAL_OK) return cleanup(rc);

  auto try_cuda = [&](cudaError_t e, const char *what) -> int {
    if (e != cudaSuccess) return galcapi::fail_cuda(e, what);
    return GAL_OK;
  };
  if ((rc = try_cuda(cudaMemset(s.chunk_ids, 0xFF, num_segments * sizeof(uint16_t)), "memset chunk_ids")) ||
      (rc = try_cuda(cudaMemset(s.seg_block_bits, 0, num_segments * s.seg_block_words * 8), "memset seg bits")) ||
      (rc = try_cuda(cudaMemset(s.block_meta, 0, nblocks * 8), "memset block_meta")) ||
      // every slice starts free; the bitmap is never rewritten afterwards
      (rc = try_cuda(cudaMemset(s.block_bits, 0xFF, nblocks * 64 * 8), "memset block_bits")) ||
      (rc = try_cuda(cudaMemset(s.locks, 0, sizeof(uint32_t)), "memset locks")) ||
      (rc = try_cuda(cudaMemset(s.nomem, 0, sizeof(uint32_t)), "memset nomem")) ||
      (rc = try_cuda(cudaMemset(s.counters, 0, GAL_NUM_COUNTERS * 8), "memset counters")) ||
      (rc = try_cuda(cudaMemset(h->d_stats, 0, 64), "memset stats")))
    return cleanup(rc);
  {
    std::vector<int32_t> gate(num_segments, (int32_t)GAL_SEG_GATE);
    if ((rc = try_cuda(cudaMemcpy(s.seg_avail, gate.data(), num_segments * 4, cudaMemcpyHostToDevice),
                       "init seg_avail")))
      return cleanup(rc);
    std::vector<uint64_t> empty(total, (uint64_t)GAL_EMPTY_BLOCK);
    if ((rc = try_cuda(cudaMemcpy(s.slots, empty.data(), total * 8, cudaMemcpyHostToDevice), "init slots")))
      return cleanup(rc);
  }
  // segment tree starts full; sub trees start empty (reference
  // gallatin.cuh:343,376-386: built full, then emptied by boot_segment_trees)
  if ((rc = galcapi::build_veb(&s.segment_tree, num_segments, seed, true, h->device_allocs)) != GAL_OK)
    return cleanup(rc);
  for (int t = 0; t < num_trees; ++t) {
    if ((rc = galcapi::build_veb(&s.sub_trees[t], num_segments, seed + (uint64_t)t, false, h->device_allocs)) !=
        GAL_OK)
      return cleanup(rc);
  }
  for (uint32_t k = 0; k < s.num_classes; ++k) {
    if ((rc = galcapi::build_veb(&s.adopt_trees[k], nblocks, seed + k, false, h->device_allocs)) != GAL_OK ||
        (rc = galcapi::build_veb(&s.roomy_trees[k], nblocks, seed + 0x100 + k, false, h->device_allocs)) != GAL_OK)
      return cleanup(rc);
  }
  if ((rc = device_alloc(h, &h->d_state, 1, "cudaMalloc state")) != GAL_OK) return cleanup(rc);
  if ((rc = try_cuda(cudaMemcpy(h->d_state, &s, sizeof(s), cudaMemcpyHostToDevice), "copy state")))
    return cleanup(rc);
  if ((rc = try_cuda(cudaDeviceSynchronize(), "create sync"))) return cleanup(rc);
  {
    std::lock_guard<std::mutex> lock(g_registry_mutex);
    g_registry[h->d_state] = h;
  }
  *out = h;
  return GAL_OK;
}

extern "C" int gal_destroy(gal_allocator *h) {
  if (h == nullptr) return fail_invalid("handle is NULL");
  cudaError_t e = cudaDeviceSynchronize();
  {
    std::lock_guard<std::mutex> lock(g_registry_mutex);
    g_registry.erase(h->d_state);
  }
  if (h->d_classes) cudaFree(h->d_classes);
  if (h->d_breqs) cudaFree(h->d_breqs);
  if (h->d_boffs) cudaFree(h->d_boffs);
  if (h->d_btable) cudaFree(h->d_btable);
  if (h->d_bsorted) cudaFree(h->d_bsorted);
  if (h->d_bbins) cudaFree(h->d_bbins);
  if (h->d_serve) cudaFree(h->d_serve);
  if (h->d_ftable) cudaFree(h->d_ftable);
  if (h->d_fused) cudaFree(h->d_fused);
  if (h->copy_event) cudaEventDestroy(h->copy_event);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  free_all(h->device_allocs);
  if (h->host_arena) cudaFreeHost(h->host_arena);
  delete h;
  if (e != cudaSuccess) return galcapi::fail_cuda(e, "destroy sync");
  return GAL_OK;
}

extern "C" void *gal_device_state(gal_allocator *h) { return h ? (void *)h->d_state : nullptr; }

extern "C" gal_allocator *gal_from_device_state(const void *device_state) {
  std::lock_guard<std::mutex> lock(g_registry_mutex);
  auto it = g_registry.find(device_state);
  return it == g_registry.end() ? nullptr : it->second;
}

extern "C" int gal_geometry(gal_allocator *h, gal_geometry_t *out) {
  if (h == nullptr || out == nullptr) return fail_invalid("NULL argument");
  const gal_state_t &s = h->hs;
  memset(out, 0, sizeof(*out));
  out->segment_bytes = s.segment_bytes;
  out->min_size = h->min_size;
  out->max_size = h->max_size;
  out->num_segments = s.num_segments;
  out->arena_bytes = s.arena_bytes;
  out->num_trees = (uint32_t)s.num_trees;
  out->blocks_per_segment = s.blocks_per_segment;
  out->num_sms = s.num_sms;
  out->total_slots = s.total_slots;
  out->num_classes = s.num_classes;
  for (uint32_t k = 0; k < s.num_classes; ++k) out->slot_count[k] = s.slot_count[k];
  out->flags = s.flags;
  out->arena_base = (uint64_t)s.memory;
  return GAL_OK;
}

extern "C" int gal_veb_layer_count(gal_allocator *h, int which, int tree) {
  if (h == nullptr) return -1;
  if (which == GAL_DUMP_SEGMENT_TREE) return h->hs.segment_tree.num_layers;
  if (which == GAL_DUMP_SUB_TREE) return (tree >= 0 && tree < h->hs.num_trees) ? h->hs.sub_trees[tree].num_layers : -1;
  if (tree < 0 || tree >= (int)h->hs.num_classes) return -1;
  if (which == GAL_DUMP_ADOPT_TREE) return h->hs.adopt_trees[tree].num_layers;
  if (which == GAL_DUMP_ROOMY_TREE) return h->hs.roomy_trees[tree].num_layers;
  return -1;
}

static bool dump_source(gal_allocator *h, int which, int tree, int layer, const void **src, uint64_t *bytes) {
  const gal_state_t &s = h->hs;
  const uint64_t nblocks = s.num_segments * s.blocks_per_segment;
  switch (which) {
    case GAL_DUMP_CHUNK_IDS: *src = s.chunk_ids; *bytes = s.num_segments * 2; return true;
    case GAL_DUMP_SEG_AVAIL: *src = s.seg_avail; *bytes = s.num_segments * 4; return true;
    case GAL_DUMP_SEG_BLOCK_BITS: *src = s.seg_block_bits; *bytes = s.num_segments * s.seg_block_words * 8; return true;
    case GAL_DUMP_BLOCK_META: *src = s.block_meta; *bytes = nblocks * 8; return true;
    case GAL_DUMP_BLOCK_BITS: *src = s.block_bits; *bytes = nblocks * 64 * 8; return true;
    case GAL_DUMP_SLOTS: *src = s.slots; *bytes = (uint64_t)s.total_slots * 8; return true;
    case GAL_DUMP_COUNTERS: *src = s.counters; *bytes = GAL_NUM_COUNTERS * 8; return true;
    case GAL_DUMP_LOCKS: *src = s.locks; *bytes = 4; return true;
    case GAL_DUMP_SEGMENT_TREE:
    case GAL_DUMP_SUB_TREE:
    case GAL_DUMP_ADOPT_TREE:
    case GAL_DUMP_ROOMY_TREE: {
      const gal_veb_t *t = nullptr;
      if (which == GAL_DUMP_SEGMENT_TREE) t = &s.segment_tree;
      else if (which == GAL_DUMP_SUB_TREE && tree >= 0 && tree < s.num_trees) t = &s.sub_trees[tree];
      else if (which == GAL_DUMP_ADOPT_TREE && tree >= 0 && tree < (int)s.num_classes) t = &s.adopt_trees[tree];
      else if (which == GAL_DUMP_ROOMY_TREE && tree >= 0 && tree < (int)s.num_classes) t = &s.roomy_trees[tree];
      if (t == nullptr || layer < 0 || layer >= t->num_layers) return false;
      *src = t->bits[layer];
      *bytes = t->layer_words[layer] * 8;
      return true;
    }
    default: return false;
  }
}

extern "C" int64_t gal_dump_bytes(gal_allocator *h, int which, int tree, int layer) {
  if (h == nullptr) return -1;
  const void *src = nullptr;
  uint64_t bytes = 0;
  if (!dump_source(h, which, tree, layer, &src, &bytes)) return -1;
  return (int64_t)bytes;
}

extern "C" int gal_dump(gal_allocator *h, int which, int tree, int layer, void *host_dst, uint64_t bytes) {
  if (h == nullptr || host_dst == nullptr) return fail_invalid("NULL argument");
  const void *src = nullptr;
  uint64_t need = 0;
  if (!dump_source(h, which, tree, layer, &src, &need)) return fail_invalid("unknown dump target");
  if (bytes < need) return fail_invalid("dump buffer too small");
  GAL_CUDA_TRY(cudaDeviceSynchronize(), "dump sync");
  GAL_CUDA_TRY(cudaMemcpy(host_dst, src, need, cudaMemcpyDeviceToHost), "dump copy");
  return GAL_OK;
}

extern "C" int gal_reset_counters(gal_allocator *h) {
  if (h == nullptr) return fail_invalid("handle is NULL");
  GAL_CUDA_TRY(cudaDeviceSynchronize(), "reset sync");
  GAL_CUDA_TRY(cudaMemset(h->hs.counters, 0, GAL_NUM_COUNTERS * 8), "reset counters");
  return GAL_OK;
}

extern "C" int gal_stats(gal_allocator *h, gal_stats_t *out) {
  if (h == nullptr || out == nullptr) return fail_invalid("NULL argument");
  const gal_state_t &s = h->hs;
  memset(out, 0, sizeof(*out));
  out->num_segments = s.num_segments;
  GAL_CUDA_TRY(cudaDeviceSynchronize(), "stats sync");
  const int leaf = s.segment_tree.num_layers - 1;
  std::vector<uint64_t> leafw(s.segment_tree.layer_words[leaf]);
  GAL_CUDA_TRY(cudaMemcpy(leafw.data(), s.segment_tree.bits[leaf], leafw.size() * 8, cudaMemcpyDeviceToHost),
               "stats copy tree");
  for (uint64_t w : leafw) out->free_segments += (uint64_t)__builtin_popcountll(w);
  std::vector<uint16_t> ids(s.num_segments);
  GAL_CUDA_TRY(cudaMemcpy(ids.data(), s.chunk_ids, ids.size() * 2, cudaMemcpyDeviceToHost), "stats copy ids");
  for (uint64_t i = 0; i < s.num_segments; ++i) {
    const uint16_t id = ids[i];
    if (id < s.num_trees) {
      out->tree_segments[id]++;
    } else if (id != GAL_FREE_SEGMENT && id > s.num_trees) {
      out->segment_allocations++;
      out->segments_in_allocations += (uint64_t)id - (uint64_t)s.num_trees - 1;
    }
  }
  const uint64_t nblocks = s.num_segments * s.blocks_per_segment;
  std::vector<uint64_t> meta(nblocks);
  GAL_CUDA_TRY(cudaMemcpy(meta.data(), s.block_meta, nblocks * 8, cudaMemcpyDeviceToHost), "stats copy meta");
  for (uint64_t m : meta) {
    const uint32_t state = (uint32_t)(m >> GAL_META_STATE_SHIFT) & 3u;
    if (state == GAL_STATE_FREE) continue;
    const uint32_t tree = (uint32_t)(m >> GAL_META_TREE_SHIFT) & 0xFFu;
    if (tree < GAL_MAX_TREES) {
      out->tree_blocks_out[tree]++;
      out->tree_live_slices[tree] += (uint32_t)m;
    }
  }
  GAL_CUDA_TRY(cudaMemcpy(out->counters, s.counters, GAL_NUM_COUNTERS * 8, cudaMemcpyDeviceToHost),
               "stats copy counters");
  return GAL_OK;
}

extern "C" int gal_print_info(gal_allocator *h) {
  gal_stats_t st;
  int rc = gal_stats(h, &st);
  if (rc != GAL_OK) return rc;
  const gal_state_t &s = h->hs;
  printf("\n\033[1;32mGallatin usage stats:\033[1;0m\n");
  printf("Segment tree sees %llu/%llu segments available\n", (unsigned long long)st.free_segments,
         (unsigned long long)st.num_segments);
  for (int t = 0; t < s.num_trees; ++t) {
    printf("Tree %d: size %llu, owns %llu/%llu, %llu blocks out, %llu live slices\n", t,
           (unsigned long long)(h->min_size << t), (unsigned long long)st.tree_segments[t],
           (unsigned long long)st.num_segments, (unsigned long long)st.tree_blocks_out[t],
           (unsigned long long)st.tree_live_slices[t]);
  }
  printf("Segment allocations: %llu spanning %llu segments\n", (unsigned long long)st.segment_allocations,
         (unsigned long long)st.segments_in_allocations);
  const uint64_t nblocks = s.num_segments * s.blocks_per_segment;
  uint64_t overhead = sizeof(gal_state_t) + s.num_segments * (2 + 4 + 8ull * s.seg_block_words) +
                      nblocks * (8 + 512) + s.total_slots * 8ull;
  printf("Allocator is using %llu bytes of overhead\n", (unsigned long long)overhead);
  printf("Counters: oom slice %llu block %llu segment %llu, timeouts %llu, bad frees %llu, corrupt %llu\n",
         (unsigned long long)st.counters[GAL_CTR_OOM_SLICE], (unsigned long long)st.counters[GAL_CTR_OOM_BLOCK],
         (unsigned long long)st.counters[GAL_CTR_OOM_SEGMENT], (unsigned long long)st.counters[GAL_CTR_TIMEOUT],
         (unsigned long long)st.counters[GAL_CTR_BAD_FREE], (unsigned long long)st.counters[GAL_CTR_CORRUPT]);
  fflush(stdout);
  return GAL_OK;
}

extern "C" int gal_set_wait_limit(gal_allocator *h, uint32_t lock_spins) {
  if (h == nullptr) return fail_invalid("handle is NULL");
  GAL_CUDA_TRY(cudaDeviceSynchronize(), "wait limit sync");
  h->hs.lock_spins = lock_spins;
  GAL_CUDA_TRY(cudaMemcpy((char *)h->d_state + offsetof(gal_state_t, lock_spins), &lock_spins, sizeof(lock_spins),
                          cudaMemcpyHostToDevice),
               "wait limit copy");
  return GAL_OK;
}

extern "C" int gal_set_locks(gal_allocator *h, uint32_t locks) {
  if (h == nullptr) return fail_invalid("handle is NULL");
  GAL_CUDA_TRY(cudaDeviceSynchronize(), "set locks sync");
  GAL_CUDA_TRY(cudaMemcpy(h->hs.locks, &locks, sizeof(locks), cudaMemcpyHostToDevice), "set locks copy");
  return GAL_OK;
}

namespace {

template <class T>
int copy_down(std::vector<T> &dst, const void *src, uint64_t count, const char *what) {
  dst.resize(count);
  if (count == 0) return GAL_OK;
  GAL_CUDA_TRY(cudaMemcpy(dst.data(), src, count * sizeof(T), cudaMemcpyDeviceToHost), what);
  return GAL_OK;
}

// Words of a vEB tree that differ from a full tree (full) or are non-zero.
int veb_diff(const gal_veb_t &t, bool full, uint64_t *diff) {
  std::vector<uint64_t> words;
  for (int layer = 0; layer < t.num_layers; ++layer) {
    int rc = copy_down(words, t.bits[layer], t.layer_words[layer], "check copy vEB layer");
    if (rc != GAL_OK) return rc;
    const uint64_t u = t.layer_universe[layer];
    for (uint64_t w = 0; w < words.size(); ++w) {
      uint64_t want = 0;
      if (full) {
        const uint64_t left = u - w * 64;
        want = left >= 64 ? ~0ull : ((1ull << left) - 1);
      }
      *diff += words[w] != want;
    }
  }
  return GAL_OK;
}

}  // namespace

extern "C" int gal_check_restored(gal_allocator *h, gal_restore_report_t *out) {
  if (h == nullptr || out == nullptr) return fail_invalid("NULL argument");
  memset(out, 0, sizeof(*out));
  const gal_state_t &s = h->hs;
  GAL_CUDA_TRY(cudaDeviceSynchronize(), "check sync");
  int rc = veb_diff(s.segment_tree, true, &out->segment_tree_words);
  for (int t = 0; rc == GAL_OK && t < s.num_trees; ++t) rc = veb_diff(s.sub_trees[t], false, &out->sub_tree_words);
  for (uint32_t k = 0; rc == GAL_OK && k < s.num_classes; ++k) {
    rc = veb_diff(s.adopt_trees[k], false, &out->adopt_tree_words);
    if (rc == GAL_OK) rc = veb_diff(s.roomy_trees[k], false, &out->adopt_tree_words);
  }
  if (rc != GAL_OK) return rc;
  std::vector<uint16_t> ids;
  if ((rc = copy_down(ids, s.chunk_ids, s.num_segments, "check copy chunk_ids")) != GAL_OK) return rc;
  for (uint16_t id : ids) out->tagged_segments += id != GAL_FREE_SEGMENT;
  std::vector<int32_t> avail;
  if ((rc = copy_down(avail, s.seg_avail, s.num_segments, "check copy seg_avail")) != GAL_OK) return rc;
  for (int32_t a : avail) out->open_segments += a != GAL_SEG_GATE;
  const uint64_t nblocks = s.num_segments * s.blocks_per_segment;
  std::vector<uint64_t> words;
  if ((rc = copy_down(words, s.block_meta, nblocks, "check copy block_meta")) != GAL_OK) return rc;
  for (uint64_t m : words) {
    out->blocks_out += ((m >> GAL_META_STATE_SHIFT) & 3u) != GAL_STATE_FREE;
    out->live_blocks += (m & GAL_META_LIVE_MASK) != 0;
  }
  // the slice bitmaps, 64 words per block, in pieces of 1 Mi words
  const uint64_t total = nblocks * GAL_BLOCK_WORDS;
  for (uint64_t at = 0; at < total; at += 1ull << 20) {
    const uint64_t n = total - at < (1ull << 20) ? total - at : (1ull << 20);
    if ((rc = copy_down(words, s.block_bits + at, n, "check copy block_bits")) != GAL_OK) return rc;
    for (uint64_t w : words) out->taken_slices += (uint64_t)__builtin_popcountll(~w);
  }
  if ((rc = copy_down(words, s.slots, s.total_slots, "check copy slots")) != GAL_OK) return rc;
  for (uint64_t v : words) out->pinned_slots += v != (uint64_t)GAL_EMPTY_BLOCK;
  std::vector<unsigned long long> ctr;
  if ((rc = copy_down(ctr, s.counters, GAL_NUM_COUNTERS, "check copy counters")) != GAL_OK) return rc;
  out->corrupt = ctr[GAL_CTR_CORRUPT];
  out->bad_frees = ctr[GAL_CTR_BAD_FREE];
  GAL_CUDA_TRY(cudaMemcpy(&out->locks, s.locks, sizeof(uint32_t), cudaMemcpyDeviceToHost), "check copy locks");
  out->restored = out->segment_tree_words == 0 && out->sub_tree_words == 0 && out->adopt_tree_words == 0 &&
                  out->tagged_segments == 0 && out->open_segments == 0 && out->blocks_out == 0 &&
                  out->live_blocks == 0 && out->taken_slices == 0 && out->pinned_slots == 0 && out->corrupt == 0 &&
                  out->bad_frees == 0 && out->locks == 0;
  return GAL_OK;
}

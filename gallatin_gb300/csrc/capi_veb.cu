// C ABI: standalone vEB tree and its ordered op runner (parity surface).
#include <cuda_runtime.h>
#include <string.h>

#include <vector>

#include "capi_internal.h"
#include "gallatin_gb300/veb.cuh"

namespace {

__device__ uint64_t run_one(const gal_veb_t *t, const gal_veb_op &op) {
  namespace v = gal::veb;
  switch (op.code) {
    case GAL_VEB_OP_INSERT: return v::insert(t, op.arg);
    case GAL_VEB_OP_INSERT_FORCE: return v::insert_force_update(t, op.arg);
    case GAL_VEB_OP_REMOVE: return v::remove(t, op.arg);
    case GAL_VEB_OP_QUERY: return v::query(t, op.arg);
    case GAL_VEB_OP_SUCCESSOR: return v::successor(t, op.arg);
    case GAL_VEB_OP_SUCCESSOR_THOROUGH: return v::successor_thorough(t, op.arg);
    case GAL_VEB_OP_LOCK_OFFSET: return v::lock_offset(t, op.arg);
    case GAL_VEB_OP_MALLOC_FIRST: return v::malloc_first(t);
    case GAL_VEB_OP_FIND_FIRST: return v::find_first_valid_index(t);
    case GAL_VEB_OP_FIND_RANDOM: return v::find_random_valid_index(t, v::thread_tid());
    case GAL_VEB_OP_MALLOC: return v::malloc_random(t, v::thread_tid());
    case GAL_VEB_OP_GATHER: return v::gather_run(t, op.arg);
    case GAL_VEB_OP_RETURN: v::return_run(t, op.arg, op.arg2); return 0;
    case GAL_VEB_OP_FIND_AT_OR_AFTER: return v::find_at_or_after(t, op.arg);
    case GAL_VEB_OP_CLAIM_FIRST: return v::claim_first(t);
    case GAL_VEB_OP_REPORT_FILL: {
      const int leaf = t->num_layers - 1;
      uint64_t fill = 0;
      for (uint64_t w = 0; w < t->layer_words[leaf]; ++w) fill += (uint64_t)__popcll(gal::ptx::ld_relaxed(t->bits[leaf] + w));
      return fill;
    }
    default: return ~0ull - 1;
  }
}

// One block of 1024 threads; op i is executed by thread ops[i].tid, so the
// hashed ops see the same thread id the reference derives from threadIdx.
__global__ void veb_ops_kernel(const gal_veb_t *t, const gal_veb_op *ops, uint64_t n, uint64_t *results) {
  for (uint64_t i = 0; i < n; ++i) {
    const gal_veb_op op = ops[i];
    if (threadIdx.x == op.tid) results[i] = run_one(t, op);
    __syncthreads();
  }
}

// ---- batched find-at-or-after -------------------------------------------
//
// Many searches on a tree nobody changes meanwhile: each CTA copies the
// tree's upper layers (as many of the top layers as fit kStageWordsMax words)
// into shared memory once, and its threads answer their queries from there;
// only the leaf words (and any upper layer too large to stage) are read from
// global memory, the leaf in aligned 128-bit pairs (every layer has an even
// number of words, the last one zero when the count is odd). The search is
// find_at_or_after's: valid when every upper bit is the OR of its child word.

constexpr unsigned kFindBlock = 512;
// 48 KiB per CTA, so four 512-thread CTAs share an SM's 227 KiB
constexpr uint64_t kStageWordsMax = 6144;

struct staged_tree {
  const uint64_t *layer[GAL_MAX_LAYERS];  // global base of each layer
  uint32_t off[GAL_MAX_LAYERS];           // shared-memory word offset of each staged layer
  uint32_t padded[GAL_MAX_LAYERS];        // words of each staged layer, padding included
  uint64_t universe;
  int num_layers;
  int staged;  // layers [0, staged) are in shared memory
};

__device__ __forceinline__ uint64_t upper_word(const staged_tree &st, const uint64_t *sm, int layer, uint64_t i) {
  return layer < st.staged ? sm[st.off[layer] + i] : __ldg(st.layer[layer] + i);
}

__device__ __forceinline__ uint64_t find_staged(const staged_tree &st, const uint64_t *sm, uint64_t x) {
  namespace v = gal::veb;
  if (x >= st.universe) return v::kFail;
  const int leaf = st.num_layers - 1;
  const uint64_t *leaf_words = st.layer[leaf];
  const uint64_t w = x >> 6;
  const ulonglong2 pr = __ldg(reinterpret_cast<const ulonglong2 *>(leaf_words + (w & ~1ull)));
  const uint64_t cur = ((w & 1) ? pr.y : pr.x) & (~0ull << (x & 63));
  if (cur) return (w << 6) + (uint64_t)(__ffsll((long long)cur) - 1);
  if (!(w & 1) && pr.y) return ((w + 1) << 6) + (uint64_t)(__ffsll((long long)pr.y) - 1);
  int layer = leaf;
  uint64_t idx = w | 1;  // search after this word of `layer`
  // on a consistent tree one float up and one float down find the answer; a
  // word found empty on the way down resumes the search after it
  for (int iter = 0; iter < 64; ++iter) {
    while (true) {
      if (layer == 0) return v::kFail;
      const uint64_t pw = idx >> 6;
      const int pb = (int)(idx & 63);
      const uint64_t bits = pb == 63 ? 0ull : (upper_word(st, sm, layer - 1, pw) & (~0ull << (pb + 1)));
      --layer;
      if (bits) {
        idx = (pw << 6) + (uint64_t)(__ffsll((long long)bits) - 1);
        ++layer;  // idx is now a word of the child layer
        break;
      }
      idx = pw;
    }
    while (true) {
      const uint64_t word = layer == leaf ? __ldg(leaf_words + idx) : upper_word(st, sm, layer, idx);
      if (word == 0) break;
      const uint64_t b = (uint64_t)(__ffsll((long long)word) - 1);
      if (layer == leaf) return (idx << 6) + b;
      idx = (idx << 6) + b;
      ++layer;
    }
  }
  return v::kFail;
}

__global__ void __launch_bounds__(kFindBlock) veb_find_staged_kernel(staged_tree st, const uint64_t *q, uint64_t n,
                                                                     uint64_t *out) {
  extern __shared__ ulonglong2 sm2[];
  uint64_t *sm = reinterpret_cast<uint64_t *>(sm2);
  for (int l = 0; l < st.staged; ++l) {
    const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(st.layer[l]);
    ulonglong2 *dst = sm2 + st.off[l] / 2;
    for (uint32_t i = threadIdx.x; i < st.padded[l] / 2; i += blockDim.x) dst[i] = __ldg(src + i);
  }
  __syncthreads();
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) out[k] = find_staged(st, sm, q[k]);
}

__global__ void veb_find_global_kernel(const gal_veb_t *t, const uint64_t *q, uint64_t n, uint64_t *out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = gal::veb::find_at_or_after(t, q[k]);
}

}  // namespace

using galcapi::fail_invalid;

extern "C" int gal_veb_create(uint64_t universe, uint64_t seed, gal_veb **out) {
  if (out == nullptr) return fail_invalid("out is NULL");
  *out = nullptr;
  gal_veb *v = new gal_veb();
  v->d_veb = nullptr;
  int rc = galcapi::build_veb(&v->hv, universe, seed, true, v->device_allocs);
  if (rc == GAL_OK) {
    cudaError_t e = cudaMalloc(&v->d_veb, sizeof(gal_veb_t));
    if (e == cudaSuccess) {
      v->device_allocs.push_back(v->d_veb);
      e = cudaMemcpy(v->d_veb, &v->hv, sizeof(gal_veb_t), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) rc = galcapi::fail_cuda(e, "vEB create");
  }
  if (rc != GAL_OK) {
    for (void *p : v->device_allocs) cudaFree(p);
    delete v;
    return rc;
  }
  *out = v;
  return GAL_OK;
}

extern "C" int gal_veb_destroy(gal_veb *v) {
  if (v == nullptr) return fail_invalid("handle is NULL");
  cudaDeviceSynchronize();
  for (void *p : v->device_allocs) cudaFree(p);
  delete v;
  return GAL_OK;
}

extern "C" int gal_veb_num_layers(gal_veb *v) { return v ? v->hv.num_layers : -1; }

extern "C" uint64_t gal_veb_layer_words(gal_veb *v, int layer) {
  if (v == nullptr || layer < 0 || layer >= v->hv.num_layers) return 0;
  return v->hv.layer_words[layer];
}

extern "C" int gal_veb_dump(gal_veb *v, int layer, uint64_t *host_dst) {
  if (v == nullptr || host_dst == nullptr || layer < 0 || layer >= v->hv.num_layers)
    return fail_invalid("bad vEB dump argument");
  GAL_CUDA_TRY(cudaDeviceSynchronize(), "vEB dump sync");
  GAL_CUDA_TRY(cudaMemcpy(host_dst, v->hv.bits[layer], v->hv.layer_words[layer] * 8, cudaMemcpyDeviceToHost),
               "vEB dump copy");
  return GAL_OK;
}

extern "C" int gal_veb_run_ops(gal_veb *v, const gal_veb_op *d_ops, uint64_t n, uint64_t *d_results,
                               void *stream) {
  if (v == nullptr || (n && (d_ops == nullptr || d_results == nullptr))) return fail_invalid("NULL argument");
  if (n == 0) return GAL_OK;
  veb_ops_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(v->d_veb, d_ops, n, d_results);
  GAL_CUDA_TRY(cudaGetLastError(), "vEB ops launch");
  return GAL_OK;
}

extern "C" int gal_veb_load(gal_veb *v, const uint64_t *host_leaf, uint64_t words) {
  if (v == nullptr || host_leaf == nullptr) return fail_invalid("NULL argument");
  const gal_veb_t &t = v->hv;
  const int leaf = t.num_layers - 1;
  if (words != t.layer_words[leaf]) return fail_invalid("leaf word count differs from the tree's");
  const uint64_t tail = t.universe & 63;
  if (tail && (host_leaf[words - 1] >> tail) != 0) return fail_invalid("a leaf bit lies past the universe");
  GAL_CUDA_TRY(cudaDeviceSynchronize(), "vEB load sync");
  std::vector<uint64_t> child(host_leaf, host_leaf + words);
  for (int layer = leaf; layer >= 0; --layer) {
    const uint64_t n = t.layer_words[layer];
    std::vector<uint64_t> cur((n + 1) & ~1ull, 0);
    if (layer == leaf) {
      for (uint64_t i = 0; i < n; ++i) cur[i] = child[i];
    } else {
      // bit b of word j: child word 64 j + b holds a set bit
      for (uint64_t c = 0; c < child.size(); ++c)
        if (child[c]) cur[c >> 6] |= 1ull << (c & 63);
    }
    GAL_CUDA_TRY(cudaMemcpy(t.bits[layer], cur.data(), cur.size() * 8, cudaMemcpyHostToDevice), "vEB load copy");
    cur.resize(n);
    child.swap(cur);
  }
  return GAL_OK;
}

extern "C" int gal_veb_find_batch(gal_veb *v, const uint64_t *d_queries, uint64_t n, uint64_t *d_out, uint32_t staged,
                                  void *stream) {
  if (v == nullptr || (n && (d_queries == nullptr || d_out == nullptr))) return fail_invalid("NULL argument");
  if (staged > 1) return fail_invalid("staged must be 0 or 1");
  if (n == 0) return GAL_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (!staged) {
    veb_find_global_kernel<<<galcapi::grid_for(n, 256), 256, 0, s>>>(v->d_veb, d_queries, n, d_out);
    GAL_CUDA_TRY(cudaGetLastError(), "vEB find launch");
    return GAL_OK;
  }
  const gal_veb_t &t = v->hv;
  staged_tree st;
  memset(&st, 0, sizeof(st));
  st.universe = t.universe;
  st.num_layers = t.num_layers;
  for (int l = 0; l < t.num_layers; ++l) st.layer[l] = t.bits[l];
  uint64_t words = 0;
  // the top layers (never the leaf) while they fit the budget
  while (st.staged < t.num_layers - 1) {
    const uint64_t padded = (t.layer_words[st.staged] + 1) & ~1ull;
    if (words + padded > kStageWordsMax) break;
    st.off[st.staged] = (uint32_t)words;
    st.padded[st.staged] = (uint32_t)padded;
    words += padded;
    ++st.staged;
  }
  const size_t smem = (size_t)words * 8;
  int dev = 0, sms = 0, per_sm = 0;
  GAL_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  GAL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
  GAL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, veb_find_staged_kernel, kFindBlock, smem),
               "occupancy query");
  if (per_sm < 1) per_sm = 1;
  uint64_t grid = (uint64_t)per_sm * sms;
  const uint64_t need = (n + kFindBlock - 1) / kFindBlock;
  if (need < grid) grid = need;
  veb_find_staged_kernel<<<(unsigned)grid, kFindBlock, smem, s>>>(st, d_queries, n, d_out);
  GAL_CUDA_TRY(cudaGetLastError(), "vEB staged find launch");
  return GAL_OK;
}

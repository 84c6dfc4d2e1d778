// ORACLE — test and baseline infrastructure only; never part of the product.
//
// C-ABI harness over the UNMODIFIED reference headers
// (saltsystemslab/gallatin include/gallatin/allocators/*.cuh), compiled by
// oracle/build.py against the copy staged in oracle/_ref/include and built
// into oracle/_ref/libgalref.so. It exposes:
//   * the reference veb_tree (veb.cuh:528-1228) behind the same ordered op
//     runner the GB300 library has, to produce golden vectors;
//   * the reference Gallatin<seg,min,max> (gallatin.cuh:292) behind the same
//     workload kernels (gallatin_gb300/csrc/workloads.cuh) the GB300 library
//     runs, for the reference arm of bench.py;
//   * its host-memory form (generate_on_device_host, gallatin.cuh:423-526)
//     paired with a device one behind the fused fill/drain kernels
//     (gallatin_gb300/csrc/spill_workloads.cuh).
#include <gallatin/allocators/gallatin.cuh>

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "gallatin_gb300.h"  // gal_veb_op layout, op codes and serving structs only
#include "ds_workloads.cuh"
#include "serving.cuh"
#include "spill_workloads.cuh"
#include "workloads.cuh"

using namespace gallatin::allocators;

namespace {

__device__ uint64_t ref_run_one(veb_tree *t, const gal_veb_op &op) {
  switch (op.code) {
    case GAL_VEB_OP_INSERT: return t->insert(op.arg);
    case GAL_VEB_OP_INSERT_FORCE: return t->insert_force_update(op.arg);
    case GAL_VEB_OP_REMOVE: return t->remove(op.arg);
    case GAL_VEB_OP_QUERY: return t->query(op.arg);
    case GAL_VEB_OP_SUCCESSOR: return t->successor(op.arg);
    case GAL_VEB_OP_SUCCESSOR_THOROUGH: return t->successor_thorough(op.arg);
    case GAL_VEB_OP_LOCK_OFFSET: return t->lock_offset(op.arg);
    case GAL_VEB_OP_MALLOC_FIRST: return t->malloc_first();
    case GAL_VEB_OP_FIND_FIRST: return t->find_first_valid_index();
    case GAL_VEB_OP_FIND_RANDOM: return t->find_random_valid_index();
    case GAL_VEB_OP_MALLOC: return t->malloc();
    case GAL_VEB_OP_GATHER: return t->gather_multiple(op.arg);
    case GAL_VEB_OP_RETURN: t->return_multiple(op.arg, op.arg2); return 0;
    case GAL_VEB_OP_REPORT_FILL: {
      layer *leaf = t->layers[t->num_layers - 1];
      uint64_t fill = 0;
      for (uint64_t w = 0; w < leaf->num_blocks; ++w) fill += (uint64_t)__popcll(leaf->bits[w]);
      return fill;
    }
    default: return ~0ull - 1;
  }
}

// op i runs on thread ops[i].tid of one 1024-thread block, so the reference's
// own threadIdx-derived tid (veb.cuh:948,996) equals ops[i].tid.
__global__ void ref_veb_ops_kernel(veb_tree *t, const gal_veb_op *ops, uint64_t n, uint64_t *results) {
  for (uint64_t i = 0; i < n; ++i) {
    const gal_veb_op op = ops[i];
    if (threadIdx.x == op.tid) results[i] = ref_run_one(t, op);
    __syncthreads();
  }
}

struct RefTree {
  veb_tree *dev;
  int num_layers;
  uint64_t words[16];
  uint64_t *bits[16];
};

using ref_16m_16_4096 = Gallatin<16ULL * 1024 * 1024, 16ULL, 4096ULL>;
using ref_16m_128_4096 = Gallatin<16ULL * 1024 * 1024, 128ULL, 4096ULL>;
using ref_64m_16_4096 = Gallatin<64ULL * 1024 * 1024, 16ULL, 4096ULL>;
using ref_4m_16_1024 = Gallatin<4ULL * 1024 * 1024, 16ULL, 1024ULL>;

struct RefAlloc {
  int config;
  void *dev;
  uint8_t *d_classes;
  uint64_t d_classes_bytes;
  unsigned long long *d_stats;
  void *d_serve;
  uint64_t d_serve_bytes;
  void *d_fused;  // device copy of the fused pair for the fused serving loop
};

int config_of(uint64_t seg, uint64_t mn, uint64_t mx) {
  if (seg == (16ull << 20) && mn == 16 && mx == 4096) return 0;
  if (seg == (16ull << 20) && mn == 128 && mx == 4096) return 1;
  if (seg == (64ull << 20) && mn == 16 && mx == 4096) return 2;
  if (seg == (4ull << 20) && mn == 16 && mx == 1024) return 3;
  return -1;
}

template <class G>
int launch_pairs(void *dev, uint64_t n, uint64_t size, uint32_t block, unsigned long long *stats, cudaStream_t s) {
  galwork::pairs_kernel<G><<<(unsigned)((n + block - 1) / block), block, 0, s>>>((G *)dev, n, size, stats);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

template <class G>
int launch_mixed(void *dev, uint64_t n, uint32_t rounds, uint64_t seed, uint32_t seg_every, uint64_t lo, uint64_t hi,
                 const uint8_t *classes, uint32_t block, unsigned long long *stats, cudaStream_t s) {
  galwork::mixed_kernel<G><<<(unsigned)((n + block - 1) / block), block, 0, s>>>((G *)dev, n, rounds, seed, seg_every,
                                                                                  lo, hi, classes, stats);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

template <class G>
int launch_batches(void *dev, const uint64_t *d_reqs, const uint64_t *d_offsets, const uint64_t *h_offsets,
                   uint32_t n_batches, uint64_t *d_table, uint32_t mode, unsigned long long *stats, cudaStream_t s) {
  G *a = (G *)dev;
  if (mode == 0) {
    for (uint32_t b = 0; b < n_batches; ++b) {
      const uint64_t n = h_offsets[b + 1] - h_offsets[b];
      if (n == 0) continue;
      galwork::batch_kernel<G><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, d_reqs + h_offsets[b], n, d_table, 32,
                                                                           stats);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
  }
  int per_sm = 0, dev_id = 0;
  cudaDeviceProp prop;
  cudaGetDevice(&dev_id);
  cudaGetDeviceProperties(&prop, dev_id);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, galwork::persistent_batches_kernel<G>, 256, 0);
  if (per_sm < 1) return 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(per_sm * prop.multiProcessorCount);
  cfg.blockDim = dim3(256);
  cfg.stream = s;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeCooperative;
  attr.val.cooperative = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  uint32_t width = 32;
  return cudaLaunchKernelEx(&cfg, galwork::persistent_batches_kernel<G>, a, d_reqs, d_offsets, n_batches, d_table,
                            width, stats) == cudaSuccess ? 0 : 2;
}

template <class G>
int launch_serving(void *dev, const galserve::server_t &sv, const galserve::trace_t &t, const galserve::params_t &p,
                   const galserve::out_t &o, cudaStream_t s) {
  int dev_id = 0;
  cudaDeviceProp prop;
  cudaGetDevice(&dev_id);
  cudaGetDeviceProperties(&prop, dev_id);
  // the plain path (mode 0): one launch per phase per step
  return galserve::run((G *)dev, sv, t, p, o, 0, 4u * prop.multiProcessorCount, s) == cudaSuccess ? 0 : 2;
}

template <class G>
int launch_fused(void *dev, void *host, uint64_t n, uint64_t seed, const uint8_t *classes, uint64_t *table,
                 uint32_t phases, unsigned long long *stats, cudaStream_t s) {
  galwork::fused_alloc<G> f{(G *)dev, (G *)host};
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (phases & 1u) galwork::fill_kernel<G><<<grid, 256, 0, s>>>(f, n, seed, classes, table, stats);
  if (phases & 2u) galwork::drain_kernel<G><<<grid, 256, 0, s>>>(f, n, seed, classes, table, stats);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

template <class G>
int launch_table(void *dev, void *heads, uint64_t nbuckets, uint64_t seed, uint32_t op, const uint64_t *keys,
                 uint64_t n, uint64_t key_seed, unsigned long long *stats, cudaStream_t s) {
  galds::chaining_table<G> t;
  t.alloc = (G *)dev;
  t.heads = (typename galds::chaining_table<G>::block_type **)heads;
  t.nbuckets = nbuckets;
  t.seed = seed;
  const uint64_t items = (op == 4 || op == 5) ? nbuckets : n;
  if (items == 0) return 0;
  galdswork::table_kernel<G><<<(unsigned)((items + 255) / 256), 256, 0, s>>>(t, keys, n, key_seed, op, stats);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

template <class G>
int launch_vectors(void *dev, const uint32_t *lengths, uint64_t n, uint32_t start, unsigned long long *stats,
                   cudaStream_t s) {
  if (n == 0) return 0;
  galdswork::vectors_kernel<G><<<(unsigned)((n + 255) / 256), 256, 0, s>>>((G *)dev, lengths, n, start, stats);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace

extern "C" {

// The same chained table and vectors (gallatin_gb300/structures.cuh) over the
// reference allocator; heads is a zeroed device array of nbuckets pointers.
int galref_table_op(void *h, void *heads, uint64_t nbuckets, uint64_t seed, uint32_t op, const uint64_t *d_keys,
                    uint64_t n, uint64_t key_seed, unsigned long long *d_stats, void *stream) {
  RefAlloc *a = (RefAlloc *)h;
  cudaStream_t s = (cudaStream_t)stream;
  switch (a->config) {
    case 0: return launch_table<ref_16m_16_4096>(a->dev, heads, nbuckets, seed, op, d_keys, n, key_seed, d_stats, s);
    case 1: return launch_table<ref_16m_128_4096>(a->dev, heads, nbuckets, seed, op, d_keys, n, key_seed, d_stats, s);
    case 2: return launch_table<ref_64m_16_4096>(a->dev, heads, nbuckets, seed, op, d_keys, n, key_seed, d_stats, s);
    default: return launch_table<ref_4m_16_1024>(a->dev, heads, nbuckets, seed, op, d_keys, n, key_seed, d_stats, s);
  }
}

int galref_run_vectors(void *h, const uint32_t *d_lengths, uint64_t n, uint32_t start, unsigned long long *d_stats,
                       void *stream) {
  RefAlloc *a = (RefAlloc *)h;
  cudaStream_t s = (cudaStream_t)stream;
  switch (a->config) {
    case 0: return launch_vectors<ref_16m_16_4096>(a->dev, d_lengths, n, start, d_stats, s);
    case 1: return launch_vectors<ref_16m_128_4096>(a->dev, d_lengths, n, start, d_stats, s);
    case 2: return launch_vectors<ref_64m_16_4096>(a->dev, d_lengths, n, start, d_stats, s);
    default: return launch_vectors<ref_4m_16_1024>(a->dev, d_lengths, n, start, d_stats, s);
  }
}

int galref_run_serving(void *h, const gal_serve_trace_t *tr, const gal_serve_params_t *pr, const gal_serve_out_t *out,
                       void *stream) {
  RefAlloc *a = (RefAlloc *)h;
  const galserve::layout_t l = galserve::layout(pr->max_slots, pr->max_pages);
  if (l.total > a->d_serve_bytes) {
    if (a->d_serve) cudaFree(a->d_serve);
    a->d_serve = nullptr;
    a->d_serve_bytes = 0;
    if (cudaMalloc(&a->d_serve, l.total) != cudaSuccess) return 3;
    a->d_serve_bytes = l.total;
  }
  const galserve::server_t sv = galserve::server_at(a->d_serve, pr->max_slots, pr->max_pages);
  galserve::trace_t t{tr->n_streams, tr->arrivals_end, tr->tokens, tr->pages, tr->page_prefix, tr->ids};
  galserve::params_t p{pr->steps, pr->tokens_per_page, pr->page_bytes, pr->budget_pages, pr->seed, 32};
  galserve::out_t o{out->checksum, out->admit_step, out->finish_step, out->step_stats,
                    (unsigned long long *)out->latency_hist};
  cudaStream_t s = (cudaStream_t)stream;
  switch (a->config) {
    case 0: return launch_serving<ref_16m_16_4096>(a->dev, sv, t, p, o, s);
    case 1: return launch_serving<ref_16m_128_4096>(a->dev, sv, t, p, o, s);
    case 2: return launch_serving<ref_64m_16_4096>(a->dev, sv, t, p, o, s);
    default: return launch_serving<ref_4m_16_1024>(a->dev, sv, t, p, o, s);
  }
}

// The serving loop with every page malloc device-first over two reference
// allocators (the second from generate_on_device_host): the reference's
// global_malloc_fused / global_free_fused pattern (global_allocator.cuh:
// 186-216) through galwork::fused_alloc. Default geometry only.
int galref_run_serving_fused(void *dev_h, void *host_h, const gal_serve_trace_t *tr, const gal_serve_params_t *pr,
                             const gal_serve_out_t *out, void *stream) {
  RefAlloc *a = (RefAlloc *)dev_h;
  RefAlloc *b = (RefAlloc *)host_h;
  if (a->config != 0 || b->config != 0) return 1;
  const galserve::layout_t l = galserve::layout(pr->max_slots, pr->max_pages);
  if (l.total > a->d_serve_bytes) {
    if (a->d_serve) cudaFree(a->d_serve);
    a->d_serve = nullptr;
    a->d_serve_bytes = 0;
    if (cudaMalloc(&a->d_serve, l.total) != cudaSuccess) return 3;
    a->d_serve_bytes = l.total;
  }
  using fused = galwork::fused_alloc<ref_16m_16_4096>;
  if (a->d_fused == nullptr && cudaMalloc(&a->d_fused, sizeof(fused)) != cudaSuccess) return 3;
  const fused f{(ref_16m_16_4096 *)a->dev, (ref_16m_16_4096 *)b->dev};
  if (cudaMemcpy(a->d_fused, &f, sizeof(f), cudaMemcpyHostToDevice) != cudaSuccess) return 2;
  const galserve::server_t sv = galserve::server_at(a->d_serve, pr->max_slots, pr->max_pages);
  galserve::trace_t t{tr->n_streams, tr->arrivals_end, tr->tokens, tr->pages, tr->page_prefix, tr->ids};
  galserve::params_t p{pr->steps, pr->tokens_per_page, pr->page_bytes, pr->budget_pages, pr->seed, 32};
  galserve::out_t o{out->checksum, out->admit_step, out->finish_step, out->step_stats,
                    (unsigned long long *)out->latency_hist};
  return launch_serving<fused>(a->d_fused, sv, t, p, o, (cudaStream_t)stream);
}

int galref_run_batches(void *h, const uint64_t *d_reqs, const uint64_t *d_offsets, const uint64_t *h_offsets,
                       uint32_t n_batches, uint64_t *d_table, uint32_t mode, unsigned long long *d_stats,
                       void *stream) {
  RefAlloc *a = (RefAlloc *)h;
  cudaStream_t s = (cudaStream_t)stream;
  switch (a->config) {
    case 0: return launch_batches<ref_16m_16_4096>(a->dev, d_reqs, d_offsets, h_offsets, n_batches, d_table, mode, d_stats, s);
    case 1: return launch_batches<ref_16m_128_4096>(a->dev, d_reqs, d_offsets, h_offsets, n_batches, d_table, mode, d_stats, s);
    case 2: return launch_batches<ref_64m_16_4096>(a->dev, d_reqs, d_offsets, h_offsets, n_batches, d_table, mode, d_stats, s);
    default: return launch_batches<ref_4m_16_1024>(a->dev, d_reqs, d_offsets, h_offsets, n_batches, d_table, mode, d_stats, s);
  }
}


int galref_veb_create(uint64_t universe, uint64_t seed, void **out) {
  RefTree *r = new RefTree();
  r->dev = veb_tree::generate_on_device(universe, seed);
  veb_tree host;
  cudaMemcpy(&host, r->dev, sizeof(veb_tree), cudaMemcpyDeviceToHost);
  r->num_layers = host.num_layers;
  layer *layer_ptrs[16];
  cudaMemcpy(layer_ptrs, host.layers, sizeof(layer *) * host.num_layers, cudaMemcpyDeviceToHost);
  for (int i = 0; i < host.num_layers; ++i) {
    layer l;
    cudaMemcpy(&l, layer_ptrs[i], sizeof(layer), cudaMemcpyDeviceToHost);
    r->words[i] = l.num_blocks;
    r->bits[i] = l.bits;
  }
  *out = r;
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
}

int galref_veb_destroy(void *h) {
  RefTree *r = (RefTree *)h;
  veb_tree::free_on_device(r->dev);
  delete r;
  return 0;
}

int galref_veb_num_layers(void *h) { return ((RefTree *)h)->num_layers; }

uint64_t galref_veb_layer_words(void *h, int layer_id) { return ((RefTree *)h)->words[layer_id]; }

int galref_veb_dump(void *h, int layer_id, uint64_t *host_dst) {
  RefTree *r = (RefTree *)h;
  cudaDeviceSynchronize();
  return cudaMemcpy(host_dst, r->bits[layer_id], r->words[layer_id] * 8, cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : 2;
}

int galref_veb_run_ops(void *h, const gal_veb_op *d_ops, uint64_t n, uint64_t *d_results, void *stream) {
  RefTree *r = (RefTree *)h;
  if (n == 0) return 0;
  ref_veb_ops_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(r->dev, d_ops, n, d_results);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

int galref_create(uint64_t max_bytes, uint64_t seed, uint64_t seg, uint64_t mn, uint64_t mx, void **out) {
  const int config = config_of(seg, mn, mx);
  if (config < 0) return 1;
  RefAlloc *a = new RefAlloc();
  a->config = config;
  a->d_classes = nullptr;
  a->d_classes_bytes = 0;
  a->d_serve = nullptr;
  a->d_serve_bytes = 0;
  a->d_fused = nullptr;
  switch (config) {
    case 0: a->dev = ref_16m_16_4096::generate_on_device(max_bytes, seed, false); break;
    case 1: a->dev = ref_16m_128_4096::generate_on_device(max_bytes, seed, false); break;
    case 2: a->dev = ref_64m_16_4096::generate_on_device(max_bytes, seed, false); break;
    default: a->dev = ref_4m_16_1024::generate_on_device(max_bytes, seed, false); break;
  }
  if (cudaMalloc(&a->d_stats, 64) != cudaSuccess) return 3;
  cudaMemset(a->d_stats, 0, 64);
  *out = a;
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
}

// The reference allocator over pinned host memory. Its generate_on_device_host
// sets cudaDeviceMapHost and exits the process if that fails
// (gallatin.cuh:437), so the flag is tried here first and a failure is
// returned instead.
int galref_create_host(uint64_t max_bytes, uint64_t seed, uint64_t seg, uint64_t mn, uint64_t mx, void **out) {
  const int config = config_of(seg, mn, mx);
  if (config < 0) return 1;
  if (cudaSetDeviceFlags(cudaDeviceMapHost) != cudaSuccess) {
    cudaGetLastError();
    return 4;
  }
  RefAlloc *a = new RefAlloc();
  a->config = config;
  a->d_classes = nullptr;
  a->d_classes_bytes = 0;
  a->d_serve = nullptr;
  a->d_serve_bytes = 0;
  a->d_fused = nullptr;
  switch (config) {
    case 0: a->dev = ref_16m_16_4096::generate_on_device_host(max_bytes, seed, false); break;
    case 1: a->dev = ref_16m_128_4096::generate_on_device_host(max_bytes, seed, false); break;
    case 2: a->dev = ref_64m_16_4096::generate_on_device_host(max_bytes, seed, false); break;
    default: a->dev = ref_4m_16_1024::generate_on_device_host(max_bytes, seed, false); break;
  }
  if (cudaMalloc(&a->d_stats, 64) != cudaSuccess) return 3;
  cudaMemset(a->d_stats, 0, 64);
  *out = a;
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
}

// Device first, host arena when the device returns NULL (the reference's
// global_malloc_fused / global_free_fused, global_allocator.cuh:186-216), in
// the fill/drain shape; dev and host must share a configuration.
int galref_run_fused(void *dev_h, void *host_h, uint64_t n, uint64_t seed, const uint8_t *d_classes,
                     uint64_t *d_table, uint32_t phases, unsigned long long *d_stats, void *stream) {
  RefAlloc *a = (RefAlloc *)dev_h;
  RefAlloc *b = (RefAlloc *)host_h;
  if (b != nullptr && b->config != a->config) return 1;
  void *host = b ? b->dev : nullptr;
  if (n == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  switch (a->config) {
    case 0: return launch_fused<ref_16m_16_4096>(a->dev, host, n, seed, d_classes, d_table, phases, d_stats, s);
    case 1: return launch_fused<ref_16m_128_4096>(a->dev, host, n, seed, d_classes, d_table, phases, d_stats, s);
    case 2: return launch_fused<ref_64m_16_4096>(a->dev, host, n, seed, d_classes, d_table, phases, d_stats, s);
    default: return launch_fused<ref_4m_16_1024>(a->dev, host, n, seed, d_classes, d_table, phases, d_stats, s);
  }
}

int galref_destroy(void *h) {
  RefAlloc *a = (RefAlloc *)h;
  cudaDeviceSynchronize();
  switch (a->config) {
    case 0: ref_16m_16_4096::free_on_device((ref_16m_16_4096 *)a->dev); break;
    case 1: ref_16m_128_4096::free_on_device((ref_16m_128_4096 *)a->dev); break;
    case 2: ref_64m_16_4096::free_on_device((ref_64m_16_4096 *)a->dev); break;
    default: ref_4m_16_1024::free_on_device((ref_4m_16_1024 *)a->dev); break;
  }
  if (a->d_classes) cudaFree(a->d_classes);
  if (a->d_serve) cudaFree(a->d_serve);
  if (a->d_fused) cudaFree(a->d_fused);
  cudaFree(a->d_stats);
  delete a;
  return 0;
}

int galref_run_pairs(void *h, uint64_t n, uint64_t size, uint32_t block, unsigned long long *d_stats, void *stream) {
  RefAlloc *a = (RefAlloc *)h;
  cudaStream_t s = (cudaStream_t)stream;
  switch (a->config) {
    case 0: return launch_pairs<ref_16m_16_4096>(a->dev, n, size, block, d_stats, s);
    case 1: return launch_pairs<ref_16m_128_4096>(a->dev, n, size, block, d_stats, s);
    case 2: return launch_pairs<ref_64m_16_4096>(a->dev, n, size, block, d_stats, s);
    default: return launch_pairs<ref_4m_16_1024>(a->dev, n, size, block, d_stats, s);
  }
}

int galref_run_mixed(void *h, uint64_t n, uint32_t rounds, uint64_t seed, uint32_t seg_every, uint64_t lo, uint64_t hi,
                     const uint8_t *d_classes, uint32_t block, unsigned long long *d_stats, void *stream) {
  RefAlloc *a = (RefAlloc *)h;
  cudaStream_t s = (cudaStream_t)stream;
  switch (a->config) {
    case 0: return launch_mixed<ref_16m_16_4096>(a->dev, n, rounds, seed, seg_every, lo, hi, d_classes, block, d_stats, s);
    case 1: return launch_mixed<ref_16m_128_4096>(a->dev, n, rounds, seed, seg_every, lo, hi, d_classes, block, d_stats, s);
    case 2: return launch_mixed<ref_64m_16_4096>(a->dev, n, rounds, seed, seg_every, lo, hi, d_classes, block, d_stats, s);
    default: return launch_mixed<ref_4m_16_1024>(a->dev, n, rounds, seed, seg_every, lo, hi, d_classes, block, d_stats, s);
  }
}

int galref_run_mixed_host(void *h, uint64_t n, uint32_t rounds, uint64_t seed, uint32_t seg_every, uint64_t lo,
                          uint64_t hi, const uint8_t *h_classes, uint32_t block, uint64_t *h_stats, void *stream) {
  RefAlloc *a = (RefAlloc *)h;
  cudaStream_t s = (cudaStream_t)stream;
  const uint64_t bytes = n * (uint64_t)rounds;
  if (bytes > a->d_classes_bytes) {
    if (a->d_classes) cudaFree(a->d_classes);
    if (cudaMalloc(&a->d_classes, bytes) != cudaSuccess) return 3;
    a->d_classes_bytes = bytes;
  }
  cudaMemsetAsync(a->d_stats, 0, 64, s);
  cudaMemcpyAsync(a->d_classes, h_classes, bytes, cudaMemcpyHostToDevice, s);
  int rc = galref_run_mixed(h, n, rounds, seed, seg_every, lo, hi, a->d_classes, block, a->d_stats, stream);
  if (rc) return rc;
  cudaMemcpyAsync(h_stats, a->d_stats, 64, cudaMemcpyDeviceToHost, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : 2;
}

}  // extern "C"

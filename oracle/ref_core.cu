// ORACLE — test and baseline infrastructure only; never part of the product.
//
// Reference harness, core family (oracle/_ref/libgalref_core.so):
//   * the reference veb_tree (veb.cuh:528-1228) behind the same ordered op
//     runner the GB300 library has, to produce golden vectors;
//   * creation and destruction of the reference Gallatin<seg,min,max>
//     (gallatin.cuh:292), on HBM and over pinned host memory
//     (generate_on_device_host, gallatin.cuh:423-526);
//   * the pairs and mixed workload kernels (gallatin_gb300/csrc/workloads.cuh)
//     over it, for the reference arm of bench.py.
#include "ref_common.cuh"
#include "workloads.cuh"

using namespace galref;

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

template <class G>
#ifndef GALREF_PAIRS_MIN_BLOCKS
#define GALREF_PAIRS_MIN_BLOCKS 1
#endif

int launch_pairs(G *dev, uint64_t n, uint64_t size, uint32_t block, unsigned long long *stats, cudaStream_t s) {
  // GALREF_PAIRS_MIN_BLOCKS=2 compiles the reference's instance for two CTAs per SM
  galwork::pairs_kernel<G, GALREF_PAIRS_MIN_BLOCKS><<<(unsigned)((n + block - 1) / block), block, 0, s>>>(dev, n, size,
                                                                                                      stats);
  return launch_status();
}

template <class G>
int launch_mixed(G *dev, uint64_t n, uint32_t rounds, uint64_t seed, uint32_t seg_every, uint64_t lo, uint64_t hi,
                 const uint8_t *classes, uint32_t block, unsigned long long *stats, cudaStream_t s) {
  galwork::mixed_kernel<G><<<(unsigned)((n + block - 1) / block), block, 0, s>>>(dev, n, rounds, seed, seg_every, lo,
                                                                                  hi, classes, stats);
  return launch_status();
}

RefAlloc *new_handle(int config) {
  RefAlloc *a = new RefAlloc();
  a->config = config;
  a->dev = nullptr;
  a->d_classes = nullptr;
  a->d_classes_bytes = 0;
  a->d_stats = nullptr;
  a->d_serve = nullptr;
  a->d_serve_bytes = 0;
  a->d_fused = nullptr;
  return a;
}

}  // namespace

extern "C" {

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
  return launch_status();
}

int galref_create(uint64_t max_bytes, uint64_t seed, uint64_t seg, uint64_t mn, uint64_t mx, void **out) {
  const int config = config_of(seg, mn, mx);
  if (config != 0 && config != 1) return 1;  // the geometries the workloads use
  RefAlloc *a = new_handle(config);
  switch (config) {
    case 0: a->dev = ref_16m_16_4096::generate_on_device(max_bytes, seed, false); break;
    case 1: a->dev = ref_16m_128_4096::generate_on_device(max_bytes, seed, false); break;
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
  if (config != 0 && config != 1) return 1;  // the geometries the workloads use
  if (cudaSetDeviceFlags(cudaDeviceMapHost) != cudaSuccess) {
    cudaGetLastError();
    return 4;
  }
  RefAlloc *a = new_handle(config);
  switch (config) {
    case 0: a->dev = ref_16m_16_4096::generate_on_device_host(max_bytes, seed, false); break;
    case 1: a->dev = ref_16m_128_4096::generate_on_device_host(max_bytes, seed, false); break;
  }
  if (cudaMalloc(&a->d_stats, 64) != cudaSuccess) return 3;
  cudaMemset(a->d_stats, 0, 64);
  *out = a;
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
}

int galref_destroy(void *h) {
  RefAlloc *a = (RefAlloc *)h;
  cudaDeviceSynchronize();
  switch (a->config) {
    case 0: ref_16m_16_4096::free_on_device((ref_16m_16_4096 *)a->dev); break;
    case 1: ref_16m_128_4096::free_on_device((ref_16m_128_4096 *)a->dev); break;
  }
  if (a->d_classes) cudaFree(a->d_classes);
  if (a->d_serve) cudaFree(a->d_serve);
  if (a->d_fused) cudaFree(a->d_fused);
  cudaFree(a->d_stats);
  delete a;
  return 0;
}

int galref_run_pairs(void *h, uint64_t n, uint64_t size, uint32_t block, unsigned long long *d_stats, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  return with_default_or_128((RefAlloc *)h, [&](auto *g) { return launch_pairs(g, n, size, block, d_stats, s); });
}

int galref_run_mixed(void *h, uint64_t n, uint32_t rounds, uint64_t seed, uint32_t seg_every, uint64_t lo, uint64_t hi,
                     const uint8_t *d_classes, uint32_t block, unsigned long long *d_stats, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  return with_default_or_128((RefAlloc *)h, [&](auto *g) {
    return launch_mixed(g, n, rounds, seed, seg_every, lo, hi, d_classes, block, d_stats, s);
  });
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

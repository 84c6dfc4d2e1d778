// ORACLE — test and baseline infrastructure only; never part of the product.
//
// Reference harness, data-structure family (oracle/_ref/libgalref_ds.so):
// the same chained hash table and doubling vectors the GB300 library runs
// (include/gallatin_gb300/structures.cuh, gallatin_gb300/csrc/
// ds_workloads.cuh) over the reference allocator. The reference's own
// chaining_table does not compile under nvcc 13 and has no delete.
#include "ref_common.cuh"
#include "ds_workloads.cuh"

using namespace galref;

namespace {

template <class G>
int launch_table(G *dev, void *heads, uint64_t nbuckets, uint64_t seed, uint32_t op, const uint64_t *keys, uint64_t n,
                 uint64_t key_seed, unsigned long long *stats, cudaStream_t s) {
  galds::chaining_table<G> t;
  t.alloc = dev;
  t.heads = (typename galds::chaining_table<G>::block_type **)heads;
  t.nbuckets = nbuckets;
  t.seed = seed;
  const uint64_t items = (op == 4 || op == 5) ? nbuckets : n;
  if (items == 0) return 0;
  galdswork::launch_table_op(t, keys, n, key_seed, op, stats, items, 256, s);
  return launch_status();
}

template <class G>
int launch_vectors(G *dev, const uint32_t *lengths, uint64_t n, uint32_t start, unsigned long long *stats,
                   cudaStream_t s) {
  if (n == 0) return 0;
  galdswork::vectors_kernel<G><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dev, lengths, n, start, stats);
  return launch_status();
}

}  // namespace

extern "C" {

// heads is a zeroed device array of nbuckets pointers.
int galref_table_op(void *h, void *heads, uint64_t nbuckets, uint64_t seed, uint32_t op, const uint64_t *d_keys,
                    uint64_t n, uint64_t key_seed, unsigned long long *d_stats, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  return with_default_or_128((RefAlloc *)h, [&](auto *g) {
    return launch_table(g, heads, nbuckets, seed, op, d_keys, n, key_seed, d_stats, s);
  });
}

int galref_run_vectors(void *h, const uint32_t *d_lengths, uint64_t n, uint32_t start, unsigned long long *d_stats,
                       void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  return with_default_or_128((RefAlloc *)h,
                             [&](auto *g) { return launch_vectors(g, d_lengths, n, start, d_stats, s); });
}

}  // extern "C"

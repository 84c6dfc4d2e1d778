// ORACLE — test and baseline infrastructure only; never part of the product.
//
// Reference harness, host-arena family (oracle/_ref/libgalref_fused.so):
// device first, host arena when the device returns NULL (the reference's
// global_malloc_fused / global_free_fused, global_allocator.cuh:186-216) in
// the fill/drain shape of gallatin_gb300/csrc/spill_workloads.cuh.
#include "ref_common.cuh"
#include "spill_workloads.cuh"

using namespace galref;

namespace {

template <class G>
int launch_fused(G *dev, void *host, uint64_t n, uint64_t seed, const uint8_t *classes, uint64_t *table,
                 uint32_t phases, unsigned long long *stats, cudaStream_t s) {
  galwork::fused_alloc<G> f{dev, (G *)host};
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (phases & 1u) galwork::fill_kernel<G><<<grid, 256, 0, s>>>(f, n, seed, classes, table, stats);
  if (phases & 2u) galwork::drain_kernel<G><<<grid, 256, 0, s>>>(f, n, seed, classes, table, stats);
  return launch_status();
}

}  // namespace

// dev and host must share a configuration; host may be NULL (device only).
extern "C" int galref_run_fused(void *dev_h, void *host_h, uint64_t n, uint64_t seed, const uint8_t *d_classes,
                                uint64_t *d_table, uint32_t phases, unsigned long long *d_stats, void *stream) {
  RefAlloc *a = (RefAlloc *)dev_h;
  RefAlloc *b = (RefAlloc *)host_h;
  if (b != nullptr && b->config != a->config) return 1;
  void *host = b ? b->dev : nullptr;
  if (n == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  return with_default(a, [&](auto *g) { return launch_fused(g, host, n, seed, d_classes, d_table, phases, d_stats, s); });
}

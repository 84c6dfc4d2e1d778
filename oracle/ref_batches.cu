// ORACLE — test and baseline infrastructure only; never part of the product.
//
// Reference harness, batching family (oracle/_ref/libgalref_batches.so): the
// batched request stream over the reference allocator through the same
// kernels the GB300 library runs (gallatin_gb300/csrc/workloads.cuh), for the
// reference arm of bench.py. The reference serves per-thread calls only, so
// its path is mode 0 (one launch per batch); mode 1 is the persistent kernel.
#include "ref_common.cuh"
#include "workloads.cuh"

using namespace galref;

namespace {

template <class G>
int launch_batches(G *a, const uint64_t *d_reqs, const uint64_t *d_offsets, const uint64_t *h_offsets,
                   uint32_t n_batches, uint64_t *d_table, uint32_t mode, unsigned long long *stats, cudaStream_t s) {
  if (mode == 0) {
    for (uint32_t b = 0; b < n_batches; ++b) {
      const uint64_t n = h_offsets[b + 1] - h_offsets[b];
      if (n == 0) continue;
      galwork::batch_kernel<G><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, d_reqs + h_offsets[b], n, d_table, 32,
                                                                           stats);
    }
    return launch_status();
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
  // one work counter per batch, zero at launch (stream-ordered scratch)
  uint32_t *work = nullptr;
  const size_t work_bytes = (size_t)n_batches * 4 + 4;
  if (cudaMallocAsync((void **)&work, work_bytes, s) != cudaSuccess) return 2;
  cudaMemsetAsync(work, 0, work_bytes, s);
  const int rc = cudaLaunchKernelEx(&cfg, galwork::persistent_batches_kernel<G>, a, d_reqs, d_offsets, n_batches,
                                    d_table, width, stats, work) == cudaSuccess ? 0 : 2;
  cudaFreeAsync(work, s);
  return rc;
}

}  // namespace

extern "C" int galref_run_batches(void *h, const uint64_t *d_reqs, const uint64_t *d_offsets,
                                  const uint64_t *h_offsets, uint32_t n_batches, uint64_t *d_table, uint32_t mode,
                                  unsigned long long *d_stats, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  return with_default((RefAlloc *)h, [&](auto *g) {
    return launch_batches(g, d_reqs, d_offsets, h_offsets, n_batches, d_table, mode, d_stats, s);
  });
}

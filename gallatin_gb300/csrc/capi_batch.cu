// C ABI: batched request streams (the batching configuration): one launch per
// batch, or one cooperative persistent launch over all batches (as given, or
// with every batch counting-sorted by size class first), optionally captured
// once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include "capi_internal.h"
#include "device_alloc.cuh"
#include "workloads.cuh"

namespace {

constexpr unsigned kBatchBlock = 256;

int grow(void **p, uint64_t *have, uint64_t need, const char *what) {
  if (need <= *have) return GAL_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *have = 0;
  GAL_CUDA_TRY(cudaMalloc(p, need), what);
  *have = need;
  return GAL_OK;
}

// u32 counters of the persistent paths: the binned path's bin counts and
// cursors (4 x kBins), then one work counter per batch.
uint64_t counter_words(uint32_t n_batches) { return 4ull * galwork::kBins + n_batches; }

// Scratch of the persistent paths: the counters, and for the binned path the
// sorted batch (sized for the largest batch). Grown before a launch or a
// capture, never inside one.
int ensure_batch_scratch(gal_allocator *h, const uint64_t *h_offsets, uint32_t n_batches, bool binned) {
  uint64_t most = 0;
  for (uint32_t b = 0; b < n_batches; ++b) {
    const uint64_t n = h_offsets[b + 1] - h_offsets[b];
    if (n > most) most = n;
  }
  // a warp takes 32 requests per atomic on a u32 counter: keep it far from wrapping
  if (most > 0x7FFFFFFFull) return galcapi::fail_invalid("a batch of the persistent paths holds at most 2^31-1 requests");
  if (binned) {
    const int rc = grow((void **)&h->d_bsorted, &h->d_bsorted_bytes, most * 8 + 8, "cudaMalloc sorted batch");
    if (rc != GAL_OK) return rc;
  }
  return grow((void **)&h->d_bbins, &h->d_bbins_bytes, counter_words(n_batches) * 4, "cudaMalloc batch counters");
}

// ctas_per_sm: kernel geometry, 0 = as many as fit (every CTA must be
// resident for the grid barrier, so more than fit is refused)
template <class K>
int launch_cooperative(gal_allocator *h, K kernel, uint32_t ctas_per_sm, cudaStream_t s, void **args) {
  int per_sm = 0;
  GAL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBatchBlock, 0), "occupancy query");
  if (per_sm < 1) return galcapi::fail_invalid("persistent batch kernel does not fit on an SM");
  if (ctas_per_sm > (uint32_t)per_sm) return galcapi::fail_invalid("more CTAs per SM than fit");
  if (ctas_per_sm) per_sm = (int)ctas_per_sm;
  GAL_CUDA_TRY(cudaLaunchCooperativeKernel((const void *)kernel, dim3(per_sm * h->hs.num_sms), dim3(kBatchBlock),
                                           args, 0, s),
               "persistent batch launch");
  return GAL_OK;
}

int launch_batches(gal_allocator *h, const uint64_t *d_reqs, const uint64_t *d_offsets, const uint64_t *h_offsets,
                   uint32_t n_batches, uint64_t *d_table, uint32_t width, uint32_t mode, uint32_t ctas_per_sm,
                   unsigned long long *d_stats, cudaStream_t s) {
  gal_device_alloc *a = reinterpret_cast<gal_device_alloc *>(h->d_state);
  if (mode == 0) {
    for (uint32_t b = 0; b < n_batches; ++b) {
      const uint64_t n = h_offsets[b + 1] - h_offsets[b];
      if (n == 0) continue;
      galwork::batch_kernel<gal_device_alloc><<<galcapi::grid_for(n, kBatchBlock), kBatchBlock, 0, s>>>(
          a, d_reqs + h_offsets[b], n, d_table, width, d_stats);
    }
    GAL_CUDA_TRY(cudaGetLastError(), "batch launch");
    return GAL_OK;
  }
  int rc = ensure_batch_scratch(h, h_offsets, n_batches, mode == 2);
  if (rc != GAL_OK) return rc;
  GAL_CUDA_TRY(cudaMemsetAsync(h->d_bbins, 0, counter_words(n_batches) * 4, s), "batch counters reset");
  uint32_t *bins = h->d_bbins;
  uint32_t *work = h->d_bbins + 4 * galwork::kBins;
  if (mode == 1) {
    void *args[] = {&a, &d_reqs, &d_offsets, &n_batches, &d_table, &width, &d_stats, &work};
    return launch_cooperative(h, galwork::persistent_batches_kernel<gal_device_alloc>, ctas_per_sm, s, args);
  }
  uint64_t *sorted = h->d_bsorted;
  void *args[] = {&a, &d_reqs, &d_offsets, &n_batches, &d_table, &width, &d_stats, &sorted, &bins, &work};
  return launch_cooperative(h, galwork::binned_batches_kernel<gal_device_alloc>, ctas_per_sm, s, args);
}

bool valid_width(uint32_t w) { return w == 8 || w == 16 || w == 32; }
constexpr const char *kModeError = "mode must be 0 (per batch), 1 (persistent) or 2 (persistent, binned)";

// Batch b is requests [offsets[b], offsets[b + 1]): the offsets must not
// decrease, or a launch would read past the request buffer. Checked on the
// host before anything is allocated or launched.
int check_offsets(const uint64_t *h_offsets, uint32_t n_batches) {
  for (uint32_t b = 0; b < n_batches; ++b)
    if (h_offsets[b + 1] < h_offsets[b]) return galcapi::fail_invalid("batch offsets must not decrease");
  return GAL_OK;
}

// The checks every batch entry point makes before it touches the GPU.
int check_batch_args(const uint64_t *h_offsets, uint32_t n_batches, uint32_t width, uint32_t mode) {
  if (!valid_width(width)) return galcapi::fail_invalid("width must be 8, 16 or 32");
  if (mode > 2) return galcapi::fail_invalid(kModeError);
  return check_offsets(h_offsets, n_batches);
}

}  // namespace

extern "C" int gal_run_batches(gal_allocator *h, const uint64_t *d_reqs, const uint64_t *d_offsets,
                               const uint64_t *h_offsets, uint32_t n_batches, uint64_t *d_table, uint32_t width,
                               uint32_t mode, uint32_t ctas_per_sm, unsigned long long *d_stats, void *stream) {
  if (h == nullptr || d_reqs == nullptr || d_offsets == nullptr || h_offsets == nullptr || d_table == nullptr ||
      d_stats == nullptr)
    return galcapi::fail_invalid("NULL argument");
  const int rc = check_batch_args(h_offsets, n_batches, width, mode);
  if (rc != GAL_OK) return rc;
  return launch_batches(h, d_reqs, d_offsets, h_offsets, n_batches, d_table, width, mode, ctas_per_sm, d_stats,
                        (cudaStream_t)stream);
}

extern "C" int gal_capture_batches(gal_allocator *h, const uint64_t *d_reqs, const uint64_t *d_offsets,
                                   const uint64_t *h_offsets, uint32_t n_batches, uint64_t *d_table, uint32_t width,
                                   uint32_t mode, uint32_t ctas_per_sm, unsigned long long *d_stats,
                                   void **graph_out) {
  if (graph_out == nullptr) return galcapi::fail_invalid("graph_out is NULL");
  *graph_out = nullptr;
  if (h == nullptr || d_reqs == nullptr || d_offsets == nullptr || h_offsets == nullptr || d_table == nullptr ||
      d_stats == nullptr)
    return galcapi::fail_invalid("NULL argument");
  if (const int rc = check_batch_args(h_offsets, n_batches, width, mode)) return rc;
  if (mode != 0) {
    const int rc = ensure_batch_scratch(h, h_offsets, n_batches, mode == 2);  // no allocation inside the capture
    if (rc != GAL_OK) return rc;
  }
  cudaStream_t s;
  GAL_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "capture stream");
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  int rc = GAL_OK;
  if (e == cudaSuccess) {
    rc = launch_batches(h, d_reqs, d_offsets, h_offsets, n_batches, d_table, width, mode, ctas_per_sm, d_stats, s);
    cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (rc == GAL_OK && e2 != cudaSuccess) rc = galcapi::fail_cuda(e2, "end capture");
  } else {
    rc = galcapi::fail_cuda(e, "begin capture");
  }
  cudaGraphExec_t exec = nullptr;
  if (rc == GAL_OK) {
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) rc = galcapi::fail_cuda(e, "graph instantiate");
  }
  if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(s);
  if (rc == GAL_OK) *graph_out = exec;
  return rc;
}

extern "C" int gal_graph_launch(void *graph_exec, void *stream) {
  if (graph_exec == nullptr) return galcapi::fail_invalid("graph is NULL");
  GAL_CUDA_TRY(cudaGraphLaunch((cudaGraphExec_t)graph_exec, (cudaStream_t)stream), "graph launch");
  return GAL_OK;
}

extern "C" int gal_graph_destroy(void *graph_exec) {
  if (graph_exec == nullptr) return GAL_OK;
  GAL_CUDA_TRY(cudaGraphExecDestroy((cudaGraphExec_t)graph_exec), "graph destroy");
  return GAL_OK;
}

extern "C" int gal_run_batches_host(gal_allocator *h, const uint64_t *h_reqs, const uint64_t *h_offsets,
                                    uint32_t n_batches, uint64_t table_slots, uint32_t width, uint32_t mode,
                                    uint32_t ctas_per_sm, uint64_t *h_stats, void *stream) {
  if (h == nullptr || h_reqs == nullptr || h_offsets == nullptr || h_stats == nullptr)
    return galcapi::fail_invalid("NULL argument");
  int rc = check_batch_args(h_offsets, n_batches, width, mode);
  if (rc != GAL_OK) return rc;
  const uint64_t nreq = h_offsets[n_batches];
  if ((rc = grow((void **)&h->d_breqs, &h->d_breqs_bytes, nreq * 8 + 8, "cudaMalloc batch requests")) ||
      (rc = grow((void **)&h->d_boffs, &h->d_boffs_bytes, (n_batches + 1) * 8ull, "cudaMalloc batch offsets")) ||
      (rc = grow((void **)&h->d_btable, &h->d_btable_bytes, table_slots * 8 + 8, "cudaMalloc batch table")))
    return rc;
  cudaStream_t s = (cudaStream_t)stream;
  GAL_CUDA_TRY(cudaMemsetAsync(h->d_stats, 0, 64, s), "stats reset");
  if (mode == 0) {
    // one launch per batch: batch b's requests are copied on a side stream
    // while the batches before it run, and its launch waits for its copy
    if (h->copy_stream == nullptr)
      GAL_CUDA_TRY(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking), "copy stream");
    if (h->copy_event == nullptr)
      GAL_CUDA_TRY(cudaEventCreateWithFlags(&h->copy_event, cudaEventDisableTiming), "copy event");
    // the copies overwrite the scratch only after earlier work on `s` that may read it
    GAL_CUDA_TRY(cudaEventRecord(h->copy_event, s), "copy event record");
    GAL_CUDA_TRY(cudaStreamWaitEvent(h->copy_stream, h->copy_event, 0), "copy stream wait");
    gal_device_alloc *a = reinterpret_cast<gal_device_alloc *>(h->d_state);
    for (uint32_t b = 0; b < n_batches; ++b) {
      const uint64_t lo = h_offsets[b], n = h_offsets[b + 1] - lo;
      if (n == 0) continue;
      GAL_CUDA_TRY(cudaMemcpyAsync(h->d_breqs + lo, h_reqs + lo, n * 8, cudaMemcpyHostToDevice, h->copy_stream),
                   "batch requests H2D");
      GAL_CUDA_TRY(cudaEventRecord(h->copy_event, h->copy_stream), "copy event record");
      GAL_CUDA_TRY(cudaStreamWaitEvent(s, h->copy_event, 0), "batch waits for its copy");
      galwork::batch_kernel<gal_device_alloc><<<galcapi::grid_for(n, kBatchBlock), kBatchBlock, 0, s>>>(
          a, h->d_breqs + lo, n, h->d_btable, width, h->d_stats);
    }
    GAL_CUDA_TRY(cudaGetLastError(), "batch launch");
    GAL_CUDA_TRY(cudaMemcpyAsync(h_stats, h->d_stats, 64, cudaMemcpyDeviceToHost, s), "stats D2H");
    GAL_CUDA_TRY(cudaStreamSynchronize(s), "batch e2e sync");
    return GAL_OK;
  }
  GAL_CUDA_TRY(cudaMemcpyAsync(h->d_breqs, h_reqs, nreq * 8, cudaMemcpyHostToDevice, s), "requests H2D");
  GAL_CUDA_TRY(cudaMemcpyAsync(h->d_boffs, h_offsets, (n_batches + 1) * 8ull, cudaMemcpyHostToDevice, s),
               "offsets H2D");
  rc = gal_run_batches(h, h->d_breqs, h->d_boffs, h_offsets, n_batches, h->d_btable, width, mode, ctas_per_sm,
                       h->d_stats, stream);
  if (rc != GAL_OK) return rc;
  GAL_CUDA_TRY(cudaMemcpyAsync(h_stats, h->d_stats, 64, cudaMemcpyDeviceToHost, s), "stats D2H");
  GAL_CUDA_TRY(cudaStreamSynchronize(s), "batch e2e sync");
  return GAL_OK;
}

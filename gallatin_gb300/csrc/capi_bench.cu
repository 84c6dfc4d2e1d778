// C ABI: the benchmark driver of the per-thread workloads (pairs, mixed).
//
// One call runs the warm-up steps, then the timed steps, each preceded by an
// L2 flush (a write of flush_bytes) and bracketed by CUDA events on the
// caller's stream, then optionally the same steps end to end through the
// host-buffer entry point with a host clock around each (class trace copied
// in, stats copied out, stream synchronised). The caller (bench.py, or any
// host program) only formats what comes back.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <chrono>

#include "capi_internal.h"

namespace {

struct scratch {
  void *flush = nullptr;
  unsigned long long *stats = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ~scratch() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (stats) cudaFree(stats);
    if (flush) cudaFree(flush);
  }
};

int launch(gal_allocator *h, const gal_bench_args_t *a, unsigned long long *d_stats) {
  if (a->workload == GAL_BENCH_PAIRS) return gal_run_pairs(h, a->n_threads, a->size, a->block_dim, d_stats, a->stream);
  return gal_run_mixed(h, a->n_threads, a->rounds, a->seed, a->seg_every, a->seg_lo, a->seg_hi, a->d_classes,
                       a->block_dim, d_stats, a->stream);
}

}  // namespace

extern "C" int gal_bench(gal_allocator *h, const gal_bench_args_t *a, gal_bench_result_t *out) {
  if (h == nullptr || a == nullptr || out == nullptr || out->step_ms == nullptr)
    return galcapi::fail_invalid("NULL argument");
  if (a->workload != GAL_BENCH_PAIRS && a->workload != GAL_BENCH_MIXED) return galcapi::fail_invalid("unknown workload");
  if (a->steps == 0) return galcapi::fail_invalid("steps must be positive");
  if (a->h_classes != nullptr && (a->workload != GAL_BENCH_MIXED || out->e2e_step_ms == nullptr))
    return galcapi::fail_invalid("the end-to-end leg needs the mixed workload and an e2e_step_ms buffer");
  cudaStream_t s = (cudaStream_t)a->stream;
  memset(out->stats, 0, sizeof(out->stats));
  memset(out->e2e_stats, 0, sizeof(out->e2e_stats));
  scratch sc;
  if (a->flush_bytes) GAL_CUDA_TRY(cudaMalloc(&sc.flush, a->flush_bytes), "cudaMalloc flush buffer");
  GAL_CUDA_TRY(cudaMalloc(&sc.stats, 8 * sizeof(unsigned long long)), "cudaMalloc bench stats");
  GAL_CUDA_TRY(cudaEventCreate(&sc.e0), "event create");
  GAL_CUDA_TRY(cudaEventCreate(&sc.e1), "event create");

  for (uint32_t i = 0; i < a->warmup; ++i) {
    int rc = launch(h, a, sc.stats);
    if (rc != GAL_OK) return rc;
  }
  GAL_CUDA_TRY(cudaStreamSynchronize(s), "warm-up sync");
  GAL_CUDA_TRY(cudaMemsetAsync(sc.stats, 0, 8 * sizeof(unsigned long long), s), "stats reset");
  for (uint32_t i = 0; i < a->steps; ++i) {
    if (sc.flush) GAL_CUDA_TRY(cudaMemsetAsync(sc.flush, (int)(i & 0xFF) | 1, a->flush_bytes, s), "L2 flush");
    GAL_CUDA_TRY(cudaEventRecord(sc.e0, s), "event record");
    int rc = launch(h, a, sc.stats);
    if (rc != GAL_OK) return rc;
    GAL_CUDA_TRY(cudaEventRecord(sc.e1, s), "event record");
    GAL_CUDA_TRY(cudaEventSynchronize(sc.e1), "event sync");
    GAL_CUDA_TRY(cudaEventElapsedTime(&out->step_ms[i], sc.e0, sc.e1), "event time");
  }
  GAL_CUDA_TRY(cudaMemcpy(out->stats, sc.stats, sizeof(out->stats), cudaMemcpyDeviceToHost), "stats copy");

  if (a->h_classes != nullptr) {
    uint64_t st[8];
    // one untimed call grows the handle's scratch for the class trace
    int rc = gal_run_mixed_host(h, a->n_threads, a->rounds, a->seed, a->seg_every, a->seg_lo, a->seg_hi,
                                a->h_classes, a->block_dim, st, a->stream);
    if (rc != GAL_OK) return rc;
    for (uint32_t i = 0; i < a->steps; ++i) {
      if (sc.flush) GAL_CUDA_TRY(cudaMemsetAsync(sc.flush, (int)(i & 0xFF) | 1, a->flush_bytes, s), "L2 flush");
      GAL_CUDA_TRY(cudaStreamSynchronize(s), "flush sync");
      const auto t0 = std::chrono::steady_clock::now();
      rc = gal_run_mixed_host(h, a->n_threads, a->rounds, a->seed, a->seg_every, a->seg_lo, a->seg_hi, a->h_classes,
                              a->block_dim, st, a->stream);
      const auto t1 = std::chrono::steady_clock::now();
      if (rc != GAL_OK) return rc;
      out->e2e_step_ms[i] = (float)std::chrono::duration<double, std::milli>(t1 - t0).count();
      for (int k = 0; k < 8; ++k) out->e2e_stats[k] += st[k];
    }
  }
  return GAL_OK;
}

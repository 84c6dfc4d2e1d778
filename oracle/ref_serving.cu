// ORACLE — test and baseline infrastructure only; never part of the product.
//
// Reference harness, serving family (oracle/_ref/libgalref_serving.so): the
// serving loop (gallatin_gb300/csrc/serving.cuh) over the reference
// allocator, on its plain path (one launch per phase per step), and over a
// device + host-memory pair of reference allocators behind the reference's
// global_malloc_fused / global_free_fused pattern (global_allocator.cuh:
// 186-216), for the reference arm of bench.py.
#include "ref_common.cuh"
#include "serving.cuh"
#include "spill_workloads.cuh"

using namespace galref;

namespace {

template <class G>
int launch_serving(G *dev, const galserve::server_t &sv, const galserve::trace_t &t, const galserve::params_t &p,
                   const galserve::out_t &o, cudaStream_t s) {
  int dev_id = 0;
  cudaDeviceProp prop;
  cudaGetDevice(&dev_id);
  cudaGetDeviceProperties(&prop, dev_id);
  // the plain path (mode 0): one launch per phase per step
  return galserve::run(dev, sv, t, p, o, 0, 4u * prop.multiProcessorCount, s) == cudaSuccess ? 0 : 2;
}

// the server's slot and page tables, owned by the handle and grown on demand
int serve_scratch(RefAlloc *a, const gal_serve_params_t *pr, galserve::server_t *out) {
  const galserve::layout_t l = galserve::layout(pr->max_slots, pr->max_pages);
  if (l.total > a->d_serve_bytes) {
    if (a->d_serve) cudaFree(a->d_serve);
    a->d_serve = nullptr;
    a->d_serve_bytes = 0;
    if (cudaMalloc(&a->d_serve, l.total) != cudaSuccess) return 3;
    a->d_serve_bytes = l.total;
  }
  *out = galserve::server_at(a->d_serve, pr->max_slots, pr->max_pages);
  return 0;
}

}  // namespace

extern "C" {

int galref_run_serving(void *h, const gal_serve_trace_t *tr, const gal_serve_params_t *pr, const gal_serve_out_t *out,
                       void *stream) {
  RefAlloc *a = (RefAlloc *)h;
  galserve::server_t sv;
  if (int rc = serve_scratch(a, pr, &sv)) return rc;
  galserve::trace_t t{tr->n_streams, tr->arrivals_end, tr->tokens, tr->pages, tr->page_prefix, tr->ids};
  galserve::params_t p{pr->steps, pr->tokens_per_page, pr->page_bytes, pr->budget_pages, pr->seed, 32};
  galserve::out_t o{out->checksum, out->admit_step, out->finish_step, out->step_stats,
                    (unsigned long long *)out->latency_hist};
  cudaStream_t s = (cudaStream_t)stream;
  return with_default(a, [&](auto *g) { return launch_serving(g, sv, t, p, o, s); });
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
  galserve::server_t sv;
  if (int rc = serve_scratch(a, pr, &sv)) return rc;
  using fused = galwork::fused_alloc<ref_16m_16_4096>;
  if (a->d_fused == nullptr && cudaMalloc(&a->d_fused, sizeof(fused)) != cudaSuccess) return 3;
  const fused f{(ref_16m_16_4096 *)a->dev, (ref_16m_16_4096 *)b->dev};
  if (cudaMemcpy(a->d_fused, &f, sizeof(f), cudaMemcpyHostToDevice) != cudaSuccess) return 2;
  galserve::trace_t t{tr->n_streams, tr->arrivals_end, tr->tokens, tr->pages, tr->page_prefix, tr->ids};
  galserve::params_t p{pr->steps, pr->tokens_per_page, pr->page_bytes, pr->budget_pages, pr->seed, 32};
  galserve::out_t o{out->checksum, out->admit_step, out->finish_step, out->step_stats,
                    (unsigned long long *)out->latency_hist};
  return launch_serving((fused *)a->d_fused, sv, t, p, o, (cudaStream_t)stream);
}

}  // extern "C"

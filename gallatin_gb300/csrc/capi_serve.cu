// C ABI: the serving loop (serving.cuh) over this allocator, with the
// server's scratch (slot tables, page tables) owned by the handle.
#include <cuda_runtime.h>

#include "capi_internal.h"
#include "device_alloc.cuh"
#include "serving.cuh"

namespace {

int check_params(const gal_serve_trace_t *tr, const gal_serve_params_t *pr, const gal_serve_out_t *out) {
  if (tr == nullptr || pr == nullptr || out == nullptr) return galcapi::fail_invalid("NULL argument");
  if (tr->arrivals_end == nullptr || tr->tokens == nullptr || tr->pages == nullptr || tr->page_prefix == nullptr)
    return galcapi::fail_invalid("trace has a NULL array");
  if (out->checksum == nullptr || out->admit_step == nullptr || out->finish_step == nullptr ||
      out->step_stats == nullptr || out->latency_hist == nullptr)
    return galcapi::fail_invalid("outputs have a NULL array");
  if (pr->steps == 0 || pr->max_slots == 0 || pr->max_pages == 0 || pr->tokens_per_page == 0)
    return galcapi::fail_invalid("steps, max_slots, max_pages and tokens_per_page must be positive");
  if (pr->tokens_per_page * 8ull > pr->page_bytes) return galcapi::fail_invalid("a page must hold its tokens (8 B each)");
  if (pr->width != 8 && pr->width != 16 && pr->width != 32) return galcapi::fail_invalid("width must be 8, 16 or 32");
  if (pr->mode > 1) return galcapi::fail_invalid("mode must be 0 (plain per-step launches) or 1 (persistent loop)");
  return GAL_OK;
}

}  // namespace

// Scratch, struct conversion and launch shared by both entry points; `a` is
// the device-side allocator object the kernels receive.
template <class A>
int run_serving_on(gal_allocator *h, A *a, const gal_serve_trace_t *tr, const gal_serve_params_t *pr,
                   const gal_serve_out_t *out, void *stream) {
  const galserve::layout_t l = galserve::layout(pr->max_slots, pr->max_pages);
  if (l.total > h->d_serve_bytes) {
    if (h->d_serve) cudaFree(h->d_serve);
    h->d_serve = nullptr;
    h->d_serve_bytes = 0;
    GAL_CUDA_TRY(cudaMalloc(&h->d_serve, l.total), "cudaMalloc serving scratch");
    h->d_serve_bytes = l.total;
  }
  const galserve::server_t sv = galserve::server_at(h->d_serve, pr->max_slots, pr->max_pages);
  galserve::trace_t t{tr->n_streams, tr->arrivals_end, tr->tokens, tr->pages, tr->page_prefix, tr->ids};
  galserve::params_t p{pr->steps, pr->tokens_per_page, pr->page_bytes, pr->budget_pages, pr->seed, pr->width};
  galserve::out_t o{out->checksum, out->admit_step, out->finish_step, out->step_stats,
                    (unsigned long long *)out->latency_hist};
  int per_sm = 0;
  GAL_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, galserve::serve_persistent_kernel<A>, 256, 0),
               "occupancy query");
  if (per_sm < 1) return galcapi::fail_invalid("serving kernel does not fit on an SM");
  if (pr->ctas_per_sm > (uint32_t)per_sm) return galcapi::fail_invalid("more CTAs per SM than fit");
  if (pr->ctas_per_sm) per_sm = (int)pr->ctas_per_sm;
  GAL_CUDA_TRY(galserve::run(a, sv, t, p, o, pr->mode, (uint32_t)per_sm * h->hs.num_sms, (cudaStream_t)stream),
               "serving launch");
  return GAL_OK;
}

extern "C" int gal_run_serving(gal_allocator *h, const gal_serve_trace_t *tr, const gal_serve_params_t *pr,
                               const gal_serve_out_t *out, void *stream) {
  if (h == nullptr) return galcapi::fail_invalid("handle is NULL");
  const int rc = check_params(tr, pr, out);
  if (rc != GAL_OK) return rc;
  return run_serving_on(h, reinterpret_cast<gal_device_alloc *>(h->d_state), tr, pr, out, stream);
}

extern "C" int gal_run_serving_fused(gal_allocator *dev, gal_allocator *host, const gal_serve_trace_t *tr,
                                     const gal_serve_params_t *pr, const gal_serve_out_t *out, void *stream) {
  if (dev == nullptr || host == nullptr) return galcapi::fail_invalid("handle is NULL");
  if (dev == host) return galcapi::fail_invalid("the host allocator must be a second allocator");
  if (dev->hs.segment_bytes != host->hs.segment_bytes)
    return galcapi::fail_invalid("both allocators must use the same segment size");
  const int rc = check_params(tr, pr, out);
  if (rc != GAL_OK) return rc;
  if (dev->d_fused == nullptr) GAL_CUDA_TRY(cudaMalloc(&dev->d_fused, sizeof(gal_fused_device_alloc)), "cudaMalloc fused");
  const gal_fused_device_alloc f{reinterpret_cast<gal_device_alloc *>(dev->d_state),
                                 reinterpret_cast<gal_device_alloc *>(host->d_state)};
  // ordered on the run's stream, after any earlier run that still reads the pair
  GAL_CUDA_TRY(cudaMemcpyAsync(dev->d_fused, &f, sizeof(f), cudaMemcpyHostToDevice, (cudaStream_t)stream),
               "fused pair H2D");
  return run_serving_on(dev, reinterpret_cast<gal_fused_device_alloc *>(dev->d_fused), tr, pr, out, stream);
}

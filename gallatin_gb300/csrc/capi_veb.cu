// C ABI: standalone vEB tree and its ordered op runner (parity surface).
#include <cuda_runtime.h>
#include <string.h>

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

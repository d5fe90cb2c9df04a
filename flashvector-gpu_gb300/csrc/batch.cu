// batch.cu -- device side of heterogeneous (served) batches.
//
// merge_main_delta_kernel is finish_delta_merge (index.rs:1353-1387) on the
// GPU: per query, the main-index answers followed by the live-insert
// ("delta") answers, entries with an invalid id dropped, a stable sort by
// distance, truncation to the query's k, padding with {u32::MAX, +inf}.
// The engine's blocking search does the same merge on the host; a served
// batch keeps it on the stream so that the batch completes without a host
// round trip.
#include <math.h>

#include "../../include/fv_bridge.h"
#include "common.cuh"
#include "kernels.h"

namespace fv {

namespace {

// One thread per query. The merged prefix is built in place in the output
// row by stable insertion: an entry goes after every kept entry whose
// distance is <= its own, and an entry that would land at position >= k is
// dropped -- the first k of the stable order, without sorting the rest.
// Both inputs are already (nearly) sorted, so each insertion moves O(1)
// entries in practice.
__global__ void merge_main_delta_kernel(const GpuSearchResult* __restrict__ main_res,
                                        const GpuSearchResult* __restrict__ delta_res, uint32_t nq, uint32_t stride,
                                        const uint32_t* __restrict__ q_topk, uint32_t top_k,
                                        GpuSearchResult* __restrict__ out) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  uint32_t k = q_topk ? __ldg(q_topk + q) : top_k;
  k = min(k, stride);
  GpuSearchResult* o = out + (size_t)q * stride;
  uint32_t n = 0;
  for (int src = 0; src < 2; ++src) {
    const GpuSearchResult* in = (src == 0 ? main_res : delta_res) + (size_t)q * stride;
    for (uint32_t r = 0; r < k; ++r) {
      const GpuSearchResult e = in[r];
      if (e.id == kInvalidId) continue;
      uint32_t j = n;
      while (j > 0 && o[j - 1].distance > e.distance) --j;
      if (j >= k) continue;
      const uint32_t last = n < k ? n : k - 1;  // the entry at k - 1 falls off when the row is full
      for (uint32_t t = last; t > j; --t) o[t] = o[t - 1];
      o[j] = e;
      if (n < k) ++n;
    }
  }
  for (uint32_t r = n; r < stride; ++r) {
    o[r].id = kInvalidId;
    o[r].distance = INFINITY;
  }
}

}  // namespace

int launch_merge_main_delta(const GpuSearchResult* main_res, const GpuSearchResult* delta_res, uint32_t nq,
                            uint32_t stride, const uint32_t* q_topk, uint32_t top_k, GpuSearchResult* out,
                            cudaStream_t stream) {
  if (nq == 0 || stride == 0) return 0;
  ProfScope ps("merge_main_delta", stream);
  merge_main_delta_kernel<<<(nq + 127) / 128, 128, 0, stream>>>(main_res, delta_res, nq, stride, q_topk, top_k, out);
  note_launch();
  return (int)cudaGetLastError();
}

}  // namespace fv

// tc_scan_fp8.cu -- instantiates the tcgen05 scan kernel for e4m3 rows
// (see tc_scan_kernel.cuh); compiled as its own translation unit so the
// precisions build in parallel.
#include "tc_scan_kernel.cuh"

namespace fv {

cudaError_t dispatch_tc_scan_fp8(int kl, int groups, int metric, bool table_scale, const CUtensorMap& ta,
                                 const CUtensorMap& tb, const TcScanArgs& a, uint32_t grid, cudaStream_t stream) {
  return dispatch_scan<true>(kl, groups, metric, table_scale, ta, tb, a, grid, stream);
}

}  // namespace fv

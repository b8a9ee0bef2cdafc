// The 128-register (MINB = 4) persistent integrate variant of one mechanism
// library, in its own translation unit so it compiles in parallel.
#include "capi_common.cuh"

namespace mkpp_tu {

int resident_blocks4() {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mkpp::integrate_persistent_kernel<Mech, 4>, mkpp::kBlock, 0);
  return std::max(1, per_sm);
}

int launch_persistent4(const mkpp::LaunchArgs& a, double* scratch, int grid, cudaStream_t stream) {
  mkpp::integrate_persistent_kernel<Mech, 4><<<grid, mkpp::kBlock, 0, stream>>>(a, scratch);
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}

}  // namespace mkpp_tu

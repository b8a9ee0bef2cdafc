// The persistent integrate kernel with tail parking (255-register variant) of
// one mechanism library, in its own translation unit so it compiles in
// parallel.  Launched instead of the plain persistent kernel when
// mkpp_set_tail_parking enables it.
#include "capi_common.cuh"

namespace mkpp_tu {

int launch_persistent_tail(const mkpp::LaunchArgs& a, double* scratch, int grid, cudaStream_t stream) {
  mkpp::integrate_persistent_kernel<Mech, 2, true><<<grid, mkpp::kBlock, 0, stream>>>(a, scratch);
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}

}  // namespace mkpp_tu

// The grid-stride (plain) integrate of one mechanism library, in its own
// translation unit so it compiles in parallel with the other kernels.
#include "capi_common.cuh"

namespace mkpp_tu {

int launch_plain(const mkpp::LaunchArgs& a, double* scratch, int grid, cudaStream_t stream) {
  mkpp::integrate_plain_kernel<Mech, 2><<<grid, mkpp::kBlock, 0, stream>>>(a, scratch);
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}

}  // namespace mkpp_tu

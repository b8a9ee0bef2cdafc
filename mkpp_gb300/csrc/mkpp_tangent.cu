// The tangent (forward sensitivity) sweep of one mechanism library, in its own
// translation unit so it compiles in parallel with the other kernels.
#include "capi_common.cuh"

namespace mkpp_tu {

int launch_tangent(const mkpp::TangentArgs& a, const mkpp::CheckpointArgs& ck, double* scratch, int grid,
                   cudaStream_t stream) {
  mkpp::tangent_kernel<Mech><<<grid, mkpp::kBlock, 0, stream>>>(a, ck, scratch);
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}

}  // namespace mkpp_tu

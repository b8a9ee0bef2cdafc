// The warp-cooperative integrate of parked cells, and the split form's
// warp-cooperative kernel, for one mechanism library, in their own
// translation unit so they compile in parallel with the other kernels.
#include "capi_common.cuh"

namespace mkpp_tu {

int set_coop_smem(size_t bytes) {
  return cudaFuncSetAttribute(mkpp::integrate_coop_kernel<Mech>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)bytes) == cudaSuccess
             ? MKPP_SUCCESS
             : MKPP_ERROR_DEVICE;
}

int launch_coop(const mkpp::LaunchArgs& a, int grid, int threads, size_t smem, cudaStream_t stream) {
  mkpp::integrate_coop_kernel<Mech><<<grid, threads, smem, stream>>>(a);
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}

int launch_split(const mkpp::LaunchArgs& a, double* scratch, int grid, cudaStream_t stream) {
  if constexpr (StoreInfo::kTile) {
    mkpp::integrate_split_kernel<Mech><<<grid, mkpp::kBlock, 0, stream>>>(a, scratch);
    return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
  } else {
    (void)a, (void)scratch, (void)grid, (void)stream;
    return MKPP_ERROR_INVALID_STATE;  // register-store mechanisms have no tile to lend the warps
  }
}

}  // namespace mkpp_tu

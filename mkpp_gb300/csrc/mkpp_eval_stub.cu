// Tendency and dense-Jacobian evaluation of a table-driven mechanism library
// (one too large for unrolled device code, such as TS1).  The evaluation
// kernels are unrolled F and J code, so these entries exist to keep the C ABI
// complete and fail with MKPP_ERROR_INVALID_STATE.
#include "capi_common.cuh"

namespace mkpp_tu {

int launch_eval_rates(size_t, const double*, const double*, double*, cudaStream_t) {
  return MKPP_ERROR_INVALID_STATE;
}

int launch_eval_jacobian(size_t, const double*, const double*, double*, cudaStream_t) {
  return MKPP_ERROR_INVALID_STATE;
}

int launch_fixed_columns(size_t, const double*, const double*, const double*, const double*, const double*,
                         const double*, double*, cudaStream_t) {
  return MKPP_ERROR_INVALID_STATE;
}

}  // namespace mkpp_tu

extern "C" {

int mkpp_gpu_evaluate_rates(size_t, const double*, const double*, double*, void*) { return MKPP_ERROR_INVALID_STATE; }

int mkpp_gpu_evaluate_jacobian(size_t, const double*, const double*, double*, void*) {
  return MKPP_ERROR_INVALID_STATE;
}

}  // extern "C"

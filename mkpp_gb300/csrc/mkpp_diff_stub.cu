// Differentiation entry points of a table-driven mechanism library (one too
// large for unrolled device code, such as TS1).  The discrete adjoint is
// generated as unrolled code only, so these entries exist to keep the C ABI
// complete and fail with MKPP_ERROR_INVALID_STATE.
#include "capi_common.cuh"

extern "C" {

size_t mkpp_gpu_adjoint_workspace_bytes(size_t) { return 0; }

int mkpp_gpu_integrate_checkpoint(size_t, double*, const double*, double, double, int, int, double*, double*, int*,
                                  int*, int*, int*, void*, size_t, void*) {
  return MKPP_ERROR_INVALID_STATE;
}

int mkpp_gpu_integrate_replay(size_t, double*, const double*, int, const double*, const int*, void*, size_t,
                              void*) {
  return MKPP_ERROR_INVALID_STATE;
}

int mkpp_gpu_adjoint(size_t, const double*, int, const double*, const double*, const int*, const double*, double*,
                     double*, void*, size_t, void*) {
  return MKPP_ERROR_INVALID_STATE;
}

}  // extern "C"

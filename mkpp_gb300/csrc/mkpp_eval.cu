// Tendency and dense-Jacobian evaluation of one mechanism library
// (compute_rates / compute_jacobian of the reference,
// src/mkpp/templates/kernel_functions/compute_{rates,jacobian}.j2).
#include "eval_common.cuh"

using namespace mkpp_tu;
using mkpp_eval::CellState;

namespace {

__global__ void __launch_bounds__(128, 1) eval_rates_kernel(size_t n, const double* conc, const double* ktab,
                                                         double* out) {
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= n) return;
  const mkpp::KTable k{ktab + c, n};
  for (int s = 0; s < Mech::NS; ++s) out[c + n * s] = 0.0;
  Mech::fun(CellState{conc, c, n}, k, [&](int i, double v) { out[c + n * Mech::var_phys(i)] = v; });
}

// Writes W slots straight into the dense (cells x N x N) LayoutLeft output.
struct DenseSlots {
  double* out;
  size_t c, n;
  __device__ __forceinline__ double& operator[](int s) const {
    return out[c + n * ((size_t)Mech::lu_prow(s) + (size_t)Mech::NS * Mech::lu_pcol(s))];
  }
};

__global__ void __launch_bounds__(128, 1) eval_jacobian_kernel(size_t n, const double* conc, const double* ktab,
                                                            double* out) {
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= n) return;
  const mkpp::KTable k{ktab + c, n};
  const size_t NS = Mech::NS;
  for (size_t e = 0; e < NS * NS; ++e) out[c + n * e] = 0.0;
  DenseSlots S{out, c, n};
  // W with inv_g_dt = 0 is -J on the W slots; flip the sign afterwards.
  Mech::jac_w(CellState{conc, c, n}, k, 0.0, S);
  Mech::for_each_w_slot([&](int slot, int, int) { S[slot] = -S[slot]; });
}

}  // namespace

namespace mkpp_tu {

int launch_eval_rates(size_t n, const double* conc, const double* ktab, double* out, cudaStream_t stream) {
  eval_rates_kernel<<<launch_grid(n, 128), 128, 0, stream>>>(n, conc, ktab, out);
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}

int launch_eval_jacobian(size_t n, const double* conc, const double* ktab, double* out, cudaStream_t stream) {
  eval_jacobian_kernel<<<launch_grid(n, 128), 128, 0, stream>>>(n, conc, ktab, out);
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}

int launch_fixed_columns(size_t n, const double* conc, const double* temp, const double* rho, const double* rh,
                         const double* clw, const double* param, double* out, cudaStream_t stream) {
  return mkpp_eval::launch_fixed_columns_kernel(n, conc, temp, rho, rh, clw, param, out, stream);
}

}  // namespace mkpp_tu

extern "C" {

int mkpp_gpu_evaluate_rates(size_t num_cells, const double* conc, const double* ktab, double* rates_out,
                            void* stream) {
  if (!conc || !ktab || !rates_out) return MKPP_ERROR_NULL_POINTER;
  if (num_cells == 0) return MKPP_ERROR_INVALID_ARGUMENT;
  return launch_eval_rates(num_cells, conc, ktab, rates_out, (cudaStream_t)stream);
}

int mkpp_gpu_evaluate_jacobian(size_t num_cells, const double* conc, const double* ktab, double* jac_out,
                               void* stream) {
  if (!conc || !ktab || !jac_out) return MKPP_ERROR_NULL_POINTER;
  if (num_cells == 0) return MKPP_ERROR_INVALID_ARGUMENT;
  eval_jacobian_kernel<<<launch_grid(num_cells, 128), 128, 0, (cudaStream_t)stream>>>(num_cells, conc, ktab,
                                                                                      jac_out);
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}


}  // extern "C"

// Tendency and dense-Jacobian evaluation of a table-driven mechanism library
// (one too large for unrolled device code, such as TS1): compute_rates /
// compute_jacobian of the reference
// (src/mkpp/templates/kernel_functions/compute_{rates,jacobian}.j2).  One
// thread per cell walks Mech::eval_step (the first stage's partials, W with
// 1/(gamma h) = 0 and F, as one sequential program) on its slice of a block
// tile, as the table-driven integrate kernels do, then writes the tendencies
// or the W-slot part of the dense Jacobian.  The tiles are allocated on the
// stream for the call.
#include "eval_common.cuh"

using namespace mkpp_tu;

namespace {

__global__ void __launch_bounds__(mkpp::kBlock, 1) eval_table_kernel(size_t n, const double* conc,
                                                                    const double* ktab, double* rates_out,
                                                                    double* jac_out, double* scratch) {
  mkpp::TileStore S{scratch + (size_t)blockIdx.x * Mech::NSLOTS * mkpp::kBlock + threadIdx.x};
  const size_t stride = (size_t)gridDim.x * mkpp::kBlock;
  const size_t NS = Mech::NS;
  for (size_t c = blockIdx.x * (size_t)mkpp::kBlock + threadIdx.x; c < n; c += stride) {
    for (int i = 0; i < Mech::NV; ++i) S[Mech::Y + i] = conc[c + n * Mech::var_phys(i)];
    const mkpp::KTable k{ktab + c, n};
    Mech::eval_step(S, k);
    if (rates_out) {
      for (size_t s = 0; s < NS; ++s) rates_out[c + n * s] = 0.0;
      for (int i = 0; i < Mech::NV; ++i) rates_out[c + n * Mech::var_phys(i)] = S[Mech::F + i];
    }
    if (jac_out) {
      for (size_t e = 0; e < NS * NS; ++e) jac_out[c + n * e] = 0.0;
      Mech::for_each_w_slot([&](int slot, int row, int col) {
        jac_out[c + n * ((size_t)row + NS * (size_t)col)] = -S[slot];
      });
    }
  }
}

int launch_table(size_t n, const double* conc, const double* ktab, double* rates_out, double* jac_out,
                 cudaStream_t stream) {
  const int grid = (int)std::min<size_t>((size_t)sm_count() * 2, (n + mkpp::kBlock - 1) / mkpp::kBlock);
  const size_t bytes = (size_t)grid * Mech::NSLOTS * mkpp::kBlock * sizeof(double);
  double* scratch = nullptr;
  if (cudaMallocAsync((void**)&scratch, bytes, stream) != cudaSuccess) return MKPP_ERROR_DEVICE;
  eval_table_kernel<<<grid, mkpp::kBlock, 0, stream>>>(n, conc, ktab, rates_out, jac_out, scratch);
  const bool launched = cudaGetLastError() == cudaSuccess;
  const bool freed = cudaFreeAsync(scratch, stream) == cudaSuccess;
  return launched && freed ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}

}  // namespace

namespace mkpp_tu {

int launch_eval_rates(size_t n, const double* conc, const double* ktab, double* out, cudaStream_t stream) {
  return launch_table(n, conc, ktab, out, nullptr, stream);
}

int launch_eval_jacobian(size_t n, const double* conc, const double* ktab, double* out, cudaStream_t stream) {
  return launch_table(n, conc, ktab, nullptr, out, stream);
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
  return launch_table(num_cells, conc, ktab, rates_out, nullptr, (cudaStream_t)stream);
}

int mkpp_gpu_evaluate_jacobian(size_t num_cells, const double* conc, const double* ktab, double* jac_out,
                               void* stream) {
  if (!conc || !ktab || !jac_out) return MKPP_ERROR_NULL_POINTER;
  if (num_cells == 0) return MKPP_ERROR_INVALID_ARGUMENT;
  return launch_table(num_cells, conc, ktab, nullptr, jac_out, (cudaStream_t)stream);
}

}  // extern "C"

// Pieces of the tendency and dense-Jacobian evaluation shared by the unrolled
// (mkpp_eval.cu) and the table-driven (mkpp_eval_table.cu) evaluation units.
// A library links exactly one of the two, so the kernel defined here exists
// once per library.
#pragma once
#include "capi_common.cuh"

namespace mkpp_eval {

// State accessor over a cell's row of the (species x cells) array.
struct CellState {
  const double* conc;
  size_t c, n;
  __device__ __forceinline__ double operator()(int i) const { return conc[c + n * Mech::var_phys(i)]; }
};

// Columns of the dense Jacobian that belong to fixed species (through the
// rate constants' dependence on them), written straight to the output.
__global__ void __launch_bounds__(128, 1) mkpp_fixed_columns_kernel(size_t n, const double* conc, const double* temp,
                                                                 const double* rho, const double* rh,
                                                                 const double* clw, const double* param,
                                                                 double* out) {
  const size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= n) return;
  const CellState y{conc, c, n};
  const double T = (Mech::RUNTIME_ENV && temp) ? temp[c] : Mech::ENV_T;
  const double RHO = (Mech::RUNTIME_ENV && rho) ? rho[c] : Mech::ENV_RHO;
  const double RH = rh ? rh[c] : 0.5;
  const double CLW = clw ? clw[c] : 0.0;
  const mkpp::CellRow fix{conc + c, n};
  const size_t NS = Mech::NS;
  auto put = [&](int row, int col, double v) { out[c + n * (row + NS * col)] = v; };
  if (param) {
    const mkpp::CellRow P{param + c, n};
    Mech::jac_fixed_columns(P, fix, T, RHO, RH, CLW, y, put);
  } else {
    const mkpp::ZeroRow P;
    Mech::jac_fixed_columns(P, fix, T, RHO, RH, CLW, y, put);
  }
}

inline int launch_fixed_columns_kernel(size_t n, const double* conc, const double* temp, const double* rho,
                                      const double* rh, const double* clw, const double* param, double* out,
                                      cudaStream_t stream) {
  mkpp_fixed_columns_kernel<<<mkpp_tu::launch_grid(n, 128), 128, 0, stream>>>(n, conc, temp, rho, rh, clw, param,
                                                                             out);
  return cudaGetLastError() == cudaSuccess ? MKPP_SUCCESS : MKPP_ERROR_DEVICE;
}

}  // namespace mkpp_eval

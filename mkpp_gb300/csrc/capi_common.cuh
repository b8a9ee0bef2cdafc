// Shared by the translation units of one mechanism library: the mechanism
// traits, launch helpers and the host functions one unit calls in another.
// Each library is built from several units compiled in parallel (integrate,
// 128-register integrate variant, differentiation, evaluation) to bound the
// compile time of the large unrolled mechanisms.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "../../include/mkpp.h"
#include "solver.cuh"
#include MKPP_MECH_HEADER

using Mech = MKPP_MECH_NS::Mech;

namespace mkpp_tu {

using StoreInfo = mkpp::StoreFor<Mech>;
constexpr size_t kQueueBytes = 256;

inline int launch_grid(size_t cells, int block) { return (int)std::max<size_t>(1, (cells + block - 1) / block); }

inline int sm_count() {
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    sms = std::max(1, sms);
  }
  return sms;
}

inline mkpp::LaunchArgs make_args(size_t cells, double* conc, const double* ktab, int steps, double dt, double seed,
                                  int max_attempts, int* status, int* accepted, int* rejected) {
  mkpp::LaunchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.ncells = (int)cells;
  a.steps = steps;
  a.dt = dt;
  a.seed = seed;
  a.max_attempts = max_attempts;
  a.conc = conc;
  a.ktab = ktab;
  a.status = status;
  a.n_accept = accepted;
  a.n_reject = rejected;
  return a;
}

// mkpp_persist4.cu: the 128-register persistent variant.
int resident_blocks4();
int launch_persistent4(const mkpp::LaunchArgs& a, double* scratch, int grid, cudaStream_t stream);
// mkpp_tail.cu: the 255-register persistent variant with tail parking.
int launch_persistent_tail(const mkpp::LaunchArgs& a, double* scratch, int grid, cudaStream_t stream);
// mkpp_eval.cu: tendency and dense-Jacobian evaluation.
int launch_eval_rates(size_t n, const double* conc, const double* ktab, double* out, cudaStream_t stream);
int launch_eval_jacobian(size_t n, const double* conc, const double* ktab, double* out, cudaStream_t stream);
int launch_fixed_columns(size_t n, const double* conc, const double* temp, const double* rho, const double* rh,
                         const double* clw, const double* param, double* out, cudaStream_t stream);
// mkpp_plain.cu: the grid-stride integrate (255-register variant).
int launch_plain(const mkpp::LaunchArgs& a, double* scratch, int grid, cudaStream_t stream);
// mkpp_coop.cu: the warp-cooperative integrate of parked cells.
int set_coop_smem(size_t bytes);
int launch_coop(const mkpp::LaunchArgs& a, int grid, int threads, size_t smem, cudaStream_t stream);
// ... and the split form (integrate_split_kernel: whole warps on reserved
// SMs, the persistent body on the others).
int launch_split(const mkpp::LaunchArgs& a, double* scratch, int grid, cudaStream_t stream);
// mkpp_checkpoint.cu, mkpp_replay.cu, mkpp_adjoint.cu: differentiation kernels.
int launch_checkpoint(const mkpp::LaunchArgs& a, const mkpp::CheckpointArgs& ck, double* scratch, int grid,
                      cudaStream_t stream);
int launch_replay(const mkpp::LaunchArgs& a, const mkpp::CheckpointArgs& ck, double* scratch, int grid,
                  cudaStream_t stream);
int launch_adjoint(const mkpp::AdjointArgs& a, const mkpp::CheckpointArgs& ck, double* scratch, int grid,
                   cudaStream_t stream);
// mkpp_tangent.cu: forward sensitivities over the recorded steps.
int launch_tangent(const mkpp::TangentArgs& a, const mkpp::CheckpointArgs& ck, double* scratch, int grid,
                   cudaStream_t stream);

}  // namespace mkpp_tu

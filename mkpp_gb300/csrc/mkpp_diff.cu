// Differentiation entry points of one mechanism library: the checkpointed
// forward, the replay of a frozen step sequence, the discrete adjoint and the
// tangent (kernels in solver.cuh, adjoint_step and tlm_step generated per
// mechanism; each kernel is launched from its own translation unit:
// mkpp_checkpoint.cu, mkpp_replay.cu, mkpp_adjoint.cu, mkpp_tangent.cu).
#include "capi_common.cuh"

using namespace mkpp_tu;

extern "C" {

// ---- Differentiation --------------------------------------------------------

static int diff_grid(size_t cells) {
  return (int)std::min<size_t>((size_t)sm_count() * 2, (cells + mkpp::kBlock - 1) / mkpp::kBlock);
}

size_t mkpp_gpu_adjoint_workspace_bytes(size_t num_cells) {
  const size_t blocks = (size_t)diff_grid(num_cells);
  const size_t fwd = mkpp::StoreN<Mech::NSLOTS>::block_bytes;
  const size_t adj = mkpp::StoreN<Mech::NSLOTS_ADJ>::block_bytes;
  return 256 + blocks * std::max(fwd, adj);
}

size_t mkpp_gpu_tangent_workspace_bytes(size_t num_cells) {
  return 256 + (size_t)diff_grid(num_cells) * Mech::NSLOTS_TLM * mkpp::kBlock * sizeof(double);
}

static int check_ckpt(size_t num_cells, int ckpt_cap, const void* a, const void* b, const void* c, const void* ws,
                      size_t ws_bytes, size_t ws_needed) {
  if (!a || !b || !c || !ws) return MKPP_ERROR_NULL_POINTER;
  if (num_cells == 0 || num_cells > (size_t)INT32_MAX || ckpt_cap < 1) return MKPP_ERROR_INVALID_ARGUMENT;
  if (ws_bytes < ws_needed) return MKPP_ERROR_INVALID_ARGUMENT;
  return MKPP_SUCCESS;
}

int mkpp_gpu_integrate_checkpoint(size_t num_cells, double* conc, const double* ktab, double dt, double seed,
                                  int max_attempts, int ckpt_cap, double* ckpt_y, double* ckpt_h, int* ckpt_n,
                                  int* status, int* accepted, int* rejected, void* workspace,
                                  size_t workspace_bytes_, void* stream) {
  int rc = check_ckpt(num_cells, ckpt_cap, ckpt_y, ckpt_h, ckpt_n, workspace, workspace_bytes_,
                      mkpp_gpu_adjoint_workspace_bytes(num_cells));
  if (rc != MKPP_SUCCESS) return rc;
  if (!conc || !ktab) return MKPP_ERROR_NULL_POINTER;
  if (!std::isfinite(dt) || dt <= 0.0 || !(seed > 0.0) || max_attempts < 1) return MKPP_ERROR_INVALID_ARGUMENT;
  mkpp::LaunchArgs a = make_args(num_cells, conc, ktab, 1, dt, seed, max_attempts, status, accepted, rejected);
  mkpp::CheckpointArgs ck{ckpt_cap, ckpt_y, ckpt_h, ckpt_n};
  double* scratch = (double*)((unsigned char*)workspace + 256);
  return launch_checkpoint(a, ck, scratch, diff_grid(num_cells), (cudaStream_t)stream);
}

int mkpp_gpu_integrate_replay(size_t num_cells, double* conc, const double* ktab, int ckpt_cap,
                              const double* ckpt_h, const int* ckpt_n, void* workspace, size_t workspace_bytes_,
                              void* stream) {
  int rc = check_ckpt(num_cells, ckpt_cap, conc, ckpt_h, ckpt_n, workspace, workspace_bytes_,
                      mkpp_gpu_adjoint_workspace_bytes(num_cells));
  if (rc != MKPP_SUCCESS) return rc;
  if (!ktab) return MKPP_ERROR_NULL_POINTER;
  mkpp::LaunchArgs a = make_args(num_cells, conc, ktab, 1, 1.0, 1.0, 1, nullptr, nullptr, nullptr);
  mkpp::CheckpointArgs ck{ckpt_cap, nullptr, const_cast<double*>(ckpt_h), const_cast<int*>(ckpt_n)};
  double* scratch = (double*)((unsigned char*)workspace + 256);
  return launch_replay(a, ck, scratch, diff_grid(num_cells), (cudaStream_t)stream);
}

int mkpp_gpu_adjoint(size_t num_cells, const double* ktab, int ckpt_cap, const double* ckpt_y,
                     const double* ckpt_h, const int* ckpt_n, const double* lambda_end, double* grad_conc0,
                     double* grad_k, void* workspace, size_t workspace_bytes_, void* stream) {
  int rc = check_ckpt(num_cells, ckpt_cap, ckpt_y, ckpt_h, ckpt_n, workspace, workspace_bytes_,
                      mkpp_gpu_adjoint_workspace_bytes(num_cells));
  if (rc != MKPP_SUCCESS) return rc;
  if (!ktab || !lambda_end || !grad_conc0 || !grad_k) return MKPP_ERROR_NULL_POINTER;
  mkpp::AdjointArgs a{(int)num_cells, ktab, lambda_end, grad_conc0, grad_k};
  mkpp::CheckpointArgs ck{ckpt_cap, const_cast<double*>(ckpt_y), const_cast<double*>(ckpt_h),
                          const_cast<int*>(ckpt_n)};
  double* scratch = (double*)((unsigned char*)workspace + 256);
  return launch_adjoint(a, ck, scratch, diff_grid(num_cells), (cudaStream_t)stream);
}

int mkpp_gpu_tangent(size_t num_cells, const double* ktab, int ckpt_cap, const double* ckpt_y,
                     const double* ckpt_h, const int* ckpt_n, const double* delta_conc0, const double* delta_k,
                     double* delta_conc, void* workspace, size_t workspace_bytes_, void* stream) {
  int rc = check_ckpt(num_cells, ckpt_cap, ckpt_y, ckpt_h, ckpt_n, workspace, workspace_bytes_,
                      mkpp_gpu_tangent_workspace_bytes(num_cells));
  if (rc != MKPP_SUCCESS) return rc;
  if (!ktab || !delta_conc0 || !delta_conc) return MKPP_ERROR_NULL_POINTER;
  mkpp::TangentArgs a{(int)num_cells, ktab, delta_conc0, delta_k, delta_conc};
  mkpp::CheckpointArgs ck{ckpt_cap, const_cast<double*>(ckpt_y), const_cast<double*>(ckpt_h),
                          const_cast<int*>(ckpt_n)};
  double* scratch = (double*)((unsigned char*)workspace + 256);
  return launch_tangent(a, ck, scratch, diff_grid(num_cells), (cudaStream_t)stream);
}


}  // extern "C"

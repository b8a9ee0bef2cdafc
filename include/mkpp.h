/*
 * mkpp.h - C ABI of one GB300-compiled MKPP mechanism library
 * (libmkpp_<mechanism>.so).
 *
 * The first block is the reference's host API, same symbols, argument meaning
 * and return codes as the header MKPP emits with `--host-api`
 * (src/mkpp/templates/host_api/mkpp.h.j2:17-72, implementation
 * src/mkpp/templates/host_api/mkpp_c_api.cpp.j2:70-374).  Like the reference,
 * the symbols are not mechanism-namespaced: one mechanism per linked library.
 * Host buffers stay caller-owned; mkpp_integrate stages them to the GPU,
 * integrates every cell there and copies the concentrations back before it
 * returns, so the call keeps the reference's blocking, in-place semantics.
 *
 * The second block (mkpp_gpu_*) has no counterpart in the reference: it takes
 * device pointers, runs on a caller-chosen CUDA stream and never blocks, for
 * host models that keep their state resident on the GPU.
 *
 * Layouts are LayoutLeft with the cell index innermost:
 *   conc[cell + num_cells * species], param[cell + num_cells * slot],
 *   jac[cell + num_cells * (row + N * col)].
 */
#ifndef MKPP_GB300_MKPP_H
#define MKPP_GB300_MKPP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Return status codes (mkpp.h.j2:17-24). */
#define MKPP_SUCCESS                  0
#define MKPP_ERROR_NULL_POINTER     -101
#define MKPP_ERROR_INVALID_HANDLE   -102
#define MKPP_ERROR_INVALID_ARGUMENT -103
#define MKPP_ERROR_INVALID_STATE    -104
#define MKPP_ERROR_CONVERGENCE      -105
#define MKPP_ERROR_NOT_FOUND        -106
/* GPU runtime failure (no reference counterpart). */
#define MKPP_ERROR_DEVICE           -107

/* Per-cell status codes written by the solver (dispatcher.hpp:15-21). */
#define MKPP_CELL_SUCCESS               0
#define MKPP_CELL_ERR_SINGULAR_MATRIX   1
#define MKPP_CELL_ERR_NON_FINITE_STATE  2
#define MKPP_CELL_ERR_CONVERGENCE       3
#define MKPP_CELL_ERR_NUMERICAL         4

typedef struct mkpp_handle_s* mkpp_handle_t;

/* ---- Reference host API (mkpp.h.j2:38-72) ---------------------------- */

/* mkpp.h.j2:38 */
int mkpp_create_handle(mkpp_handle_t* handle_out, size_t num_cells);
/* mkpp.h.j2:39 */
int mkpp_destroy_handle(mkpp_handle_t handle);
/* mkpp.h.j2:40 */
int mkpp_initialize(mkpp_handle_t handle);
/* mkpp.h.j2:43-47 */
int mkpp_get_species_count(mkpp_handle_t handle, size_t* count_out);
int mkpp_get_reaction_count(mkpp_handle_t handle, size_t* count_out);
int mkpp_get_photolysis_count(mkpp_handle_t handle, size_t* count_out);
int mkpp_get_species_index(mkpp_handle_t handle, const char* species_name, int* index_out);
int mkpp_get_photolysis_index(mkpp_handle_t handle, const char* photo_name, int* index_out);
/* mkpp.h.j2:50-54: LayoutLeft (cells x species) concentrations, per-cell T, p, rho. */
int mkpp_set_state_ptrs(mkpp_handle_t handle, double* species_conc, const double* temp,
                        const double* pressure, const double* air_density);
/* mkpp.h.j2:57: values[cell + num_cells * parameter]; count must equal the
 * mechanism's runtime parameter count. */
int mkpp_set_rate_parameter_ptrs(mkpp_handle_t handle, const double* values, size_t count);
/* mkpp.h.j2:59 */
int mkpp_set_photolysis_ptrs(mkpp_handle_t handle, const double* photolysis_rates);
/* mkpp.h.j2:61 */
int mkpp_set_cloud_water_ptr(mkpp_handle_t handle, const double* values);
/* mkpp.h.j2:63-65 */
int mkpp_set_aerosol_ptrs(mkpp_handle_t handle, const double* relative_humidity,
                          const double* aerosol_surface_area);
/* mkpp.h.j2:68: integrates every cell over dt seconds, in place. */
int mkpp_integrate(mkpp_handle_t handle, double dt);
/* mkpp.h.j2:70: species tendencies, (cells x species) LayoutLeft. */
int mkpp_evaluate_rates(mkpp_handle_t handle, double* rates_out);
/* mkpp.h.j2:71: dense Jacobian (cells x N x N) LayoutLeft. */
int mkpp_evaluate_jacobian(mkpp_handle_t handle, double* jac_out);
/* Products with that Jacobian, the per-cell quantities of the reference's
 * SolverKernels::compute_tlm (dF = J delta,
 * src/mkpp/templates/kernel_functions/compute_tlm.j2) and compute_adjoint
 * (J^T, compute_adjoint.j2) applied to a vector: out = J delta or J^T lambda,
 * all (cells x species) LayoutLeft host arrays (no reference C entry). */
int mkpp_evaluate_jacobian_vector(mkpp_handle_t handle, const double* delta, double* out);
int mkpp_evaluate_jacobian_transpose_vector(mkpp_handle_t handle, const double* lambda, double* out);
/* mkpp.h.j2:74 */
int mkpp_get_last_error(mkpp_handle_t handle, char* buffer, size_t buffer_len);

/* ---- Handle options (no reference C entry; the reference exposes the
 * seed as the SolverKernels::initial_step_seed member, integrate.j2:42) --- */
int mkpp_set_initial_step_seed(mkpp_handle_t handle, double seed);
/* Upper bound on attempts per integrate() call (default 20000); a cell that
 * reaches it reports MKPP_CELL_ERR_CONVERGENCE. */
int mkpp_set_max_attempts(mkpp_handle_t handle, int max_attempts);
/* Read back the per-cell status / accepted / rejected counts of the last
 * mkpp_integrate (each array num_cells ints; any may be NULL).  A cell
 * skipped because its input is not finite (status 2) reports 0 accepted
 * and 0 rejected steps for that call. */
int mkpp_get_cell_stats(mkpp_handle_t handle, int* status, int* accepted, int* rejected);
/* Cost ordering (default on): each mkpp_integrate hands out first the cells
 * that needed the most attempts in the previous call on this handle, so the
 * slowest cells start first and the call's tail shrinks.  Results do not
 * depend on it (cells are independent); it reads back num_cells x 2 ints per
 * call and sends the order (num_cells ints).  enable 0 turns it off and
 * forgets the counts. */
int mkpp_set_cost_order(mkpp_handle_t handle, int enable);
/* Step-size carry-over (default off; no reference entry: the reference
 * restarts every integrate() at dt * initial_step_seed and lists carried
 * step estimates as future work, SCALING_OPTIMIZATION_REPORT.md:27-29).
 * When on, each mkpp_integrate starts every cell at the step size its
 * previous call on this handle ended with (the controller's proposal after
 * the last accepted step, or the step wanted before a last step cut short to
 * end at dt), the first call after enabling at dt * seed.  It changes the
 * step sequence, so results differ from the reference's within the
 * tolerances; it removes the ramp from dt * seed at every call. */
int mkpp_set_dt_carryover(mkpp_handle_t handle, int enable);

/* ---- Mechanism metadata (no reference C entry; compile-time constants of
 * the generated SolverKernels, header.j2:127-186) ------------------------ */
int mkpp_mechanism_name(const char** name_out);
/* species, variable species, reactions, runtime parameter slots, LU slots */
int mkpp_mechanism_sizes(int* num_species, int* num_variable, int* num_reactions,
                         int* num_rate_parameters, int* num_lu_slots);
/* SUPPORTS_RUNTIME_ENVIRONMENT and HAS_CLOUD_GATED of the reference's
 * SolverKernels (header.j2:127-186) as 0/1; either pointer may be NULL. */
int mkpp_mechanism_flags(int* runtime_environment, int* cloud_gated);
/* SolverKernels::atol[] / rtol[]: NS values each, physical species order;
 * either pointer may be NULL. */
int mkpp_mechanism_tolerances(double* atol, double* rtol);

/* ---- Device-pointer entry points (no reference counterpart) ----------- */

/* Workspace bytes mkpp_gpu_integrate_k / _logged need for num_cells cells:
 * work counters, the per-block LU/stage scratch tiles of the integrate grid
 * and one parked-cell record per cell.  Depends on the launch tuning: query it
 * after mkpp_set_launch_tuning.  The workspace must be 256-byte aligned. */
size_t mkpp_gpu_workspace_bytes(size_t num_cells);

/* Process-wide launch tuning of the integrate kernels (the autotuner's
 * knobs): register_variant 2 (up to 255 registers per thread) or 4 (up to
 * 128, more resident warps), 0 keeps the current one; blocks_per_sm caps the
 * resident blocks per SM (0: as many as fit); defer_after: attempts per host
 * step of a launch (a launch over S steps: defer_after * S in all) after which
 * the persistent kernel hands a cell to the warp-cooperative kernel (0: never,
 * -1 keeps the current value; default 3000, environment MKPP_DEFER_AFTER).
 * Results do not depend on it: a handed-off cell ends bit-identical. */
int mkpp_set_launch_tuning(int register_variant, int blocks_per_sm, int defer_after);

/* Process-wide tail parking of the persistent integrate kernel (default 300
 * attempts, 0: off; environment MKPP_TAIL_AFTER).  Once every cell of a launch has been
 * handed out and no more cells are still on lanes than the warp-cooperative
 * kernel runs at once, a cell with at least min_attempts attempts is parked
 * for that kernel, which takes a warp per cell.  The last, slowest cells of a
 * call then finish faster.  Results do not depend on it: a parked cell ends
 * bit-identical.  Applies to the 255-register variant. */
int mkpp_set_tail_parking(int min_attempts);
/* Split launch (process-wide, default off; no reference counterpart): when
 * a persistent integrate launch has a cell_order, the blocks on the first
 * split_sms SMs integrate its first split_cells cells, each on a whole warp
 * (the warp-cooperative attempt), while the other SMs run the persistent
 * kernel's body over the rest of the order, in the same launch.  A warp on
 * an SM that runs no lanes finishes an attempt of one cell about 3x sooner
 * than a lane, so the few most expensive cells, which otherwise set the end
 * of the launch, finish earlier.  Results are bit-identical.  Applies to the
 * 255-register variant without tail parking.  Give the cells in cost order
 * (most expensive first), e.g. the previous window's attempt counts. */
int mkpp_set_split_launch(int split_cells, int split_sms);

/* Rate constants of every reaction into ktab[cell + num_cells * reaction].
 * temp/rho/rh/clw/param may be NULL (compile-time environment, 0.5, 0, zeros).
 * status (may be NULL) receives MKPP_CELL_ERR_NON_FINITE_STATE for cells with
 * non-finite inputs, MKPP_CELL_SUCCESS otherwise. */
int mkpp_gpu_rate_constants(size_t num_cells, const double* conc, const double* temp,
                            const double* rho, const double* rh, const double* clw,
                            const double* param, size_t num_params, double* ktab,
                            int* status, void* stream);

/* Integrate every cell over `steps` consecutive host steps of dt seconds
 * from precomputed rate constants: host step s reads the rate table at
 * ktab + s * k_step_stride (k_step_stride = 0: the same rate constants for
 * every step, like the reference's repeated integrate() calls; otherwise at
 * least num_cells * reactions).  A cell runs through all its host steps
 * before its thread takes the next cell.
 * mode 0 = one thread per cell (plain), 1 = persistent work queue.
 * cell_order (mode 1, may be NULL): a permutation of the cells giving the
 * order in which the queue hands them out, e.g. most expensive first.
 * workspace: at least mkpp_gpu_workspace_bytes(num_cells) bytes of device
 * memory (queue counter and per-block scratch).  Cells whose status is
 * non-zero on entry are skipped; on exit status holds each cell's outcome
 * (MKPP_CELL_*).  Asynchronous on `stream`. */
int mkpp_gpu_integrate_k(size_t num_cells, double* conc, const double* ktab,
                         size_t k_step_stride, int steps, double dt, double seed,
                         int max_attempts, int mode,
                         const int* cell_order, int* status, int* accepted, int* rejected,
                         void* workspace, size_t workspace_bytes, void* stream);

/* mkpp_gpu_integrate_k with step-size carry-over (see mkpp_set_dt_carryover):
 * dt_carry [num_cells] doubles on the device, in/out.  dt_carry[c] > 0 starts
 * cell c's first call at that step size (0: at dt * seed), later calls of the
 * launch start from the previous call's carry, and the last one is written
 * back.  No reference counterpart. */
int mkpp_gpu_integrate_carry(size_t num_cells, double* conc, const double* ktab,
                             size_t k_step_stride, int steps, double dt, double seed,
                             int max_attempts, int mode, const int* cell_order, int* status,
                             int* accepted, int* rejected, double* dt_carry, void* workspace,
                             size_t workspace_bytes, void* stream);

/* Same as mkpp_gpu_integrate_k, also recording every attempt's step size and
 * accept flag (log_h/log_acc[attempt * num_cells + cell], log_n[cell]) for
 * step-sequence replay; plain mode only. */
int mkpp_gpu_integrate_logged(size_t num_cells, double* conc, const double* ktab, int steps,
                              double dt, double seed, int max_attempts, int* status,
                              int* accepted, int* rejected, double* log_h,
                              unsigned char* log_acc, int* log_n, int log_cap, void* workspace,
                              size_t workspace_bytes, void* stream);

/* Species tendencies F (LayoutLeft cells x N, fixed species 0) from rate constants. */
int mkpp_gpu_evaluate_rates(size_t num_cells, const double* conc, const double* ktab,
                            double* rates_out, void* stream);
/* Dense Jacobian (cells x N x N LayoutLeft, fixed rows and columns 0). */
int mkpp_gpu_evaluate_jacobian(size_t num_cells, const double* conc, const double* ktab,
                               double* jac_out, void* stream);

/* ---- Differentiation (discrete adjoint; the reference's counterparts are
 * SolverKernels::integrate_fwd_checkpoint / integrate_adj,
 * src/mkpp/templates/solver_variants/integrate_fwd_checkpoint.j2:36-295 and
 * integrate_adj.j2:49-156, a frozen-Jacobian reverse sweep; this one is the
 * full discrete adjoint of the accepted steps, with the Jacobian's
 * dependence on the state and on the rate constants) ------------------- */
#define MKPP_CELL_ERR_CHECKPOINT_OVERFLOW 5
/* Workspace of the three calls below (per-thread scratch, 256-byte aligned). */
size_t mkpp_gpu_adjoint_workspace_bytes(size_t num_cells);
/* One integrate() call over dt (same controller and arithmetic as the plain
 * form) that records, at every accepted step s < ckpt_cap, the state before
 * the step at ckpt_y[(s * NV + i) * num_cells + cell] (NV variable species in
 * the solver's order) and the step size at ckpt_h[s * num_cells + cell];
 * ckpt_n[cell] = accepted steps.  More accepted steps than ckpt_cap:
 * MKPP_CELL_ERR_CHECKPOINT_OVERFLOW. */
int mkpp_gpu_integrate_checkpoint(size_t num_cells, double* conc, const double* ktab, double dt,
                                  double seed, int max_attempts, int ckpt_cap, double* ckpt_y,
                                  double* ckpt_h, int* ckpt_n, int* status, int* accepted,
                                  int* rejected, void* workspace, size_t workspace_bytes, void* stream);
/* Applies the recorded step sizes (frozen step sequence) to conc. */
int mkpp_gpu_integrate_replay(size_t num_cells, double* conc, const double* ktab, int ckpt_cap,
                              const double* ckpt_h, const int* ckpt_n, void* workspace,
                              size_t workspace_bytes, void* stream);
/* Given lambda_end = dL/dconc at the end of the checkpointed call
 * ([species][cells]), writes dL/dconc at its start (fixed species 0) and
 * dL/dk ([reactions][cells]) for the recorded step sequence. */
int mkpp_gpu_adjoint(size_t num_cells, const double* ktab, int ckpt_cap, const double* ckpt_y,
                     const double* ckpt_h, const int* ckpt_n, const double* lambda_end,
                     double* grad_conc0, double* grad_k, void* workspace, size_t workspace_bytes,
                     void* stream);

/* ---- Tangent (forward sensitivities; the reference's counterpart is
 * SolverKernels::integrate_tlm, src/mkpp/templates/solver_variants/
 * integrate_tlm.j2:32-215, a frozen-Jacobian tangent in the state alone;
 * this one is the exact tangent of the accepted steps, the transpose of
 * mkpp_gpu_adjoint, and also carries a direction in the rate constants) --- */
/* Workspace of mkpp_gpu_tangent (per-thread scratch, 256-byte aligned). */
size_t mkpp_gpu_tangent_workspace_bytes(size_t num_cells);
/* Given the checkpoints of mkpp_gpu_integrate_checkpoint, a direction
 * delta_conc0 in the starting state ([species][cells]; fixed species
 * ignored) and delta_k in the rate constants ([reactions][cells], or NULL
 * for none), writes delta_conc = d conc_end / d (conc0, k) applied to them
 * ([species][cells]; fixed species 0) for the recorded step sequence. */
int mkpp_gpu_tangent(size_t num_cells, const double* ktab, int ckpt_cap, const double* ckpt_y,
                     const double* ckpt_h, const int* ckpt_n, const double* delta_conc0,
                     const double* delta_k, double* delta_conc, void* workspace,
                     size_t workspace_bytes, void* stream);

/* Allocation-free integrate (no counterpart in the reference).  For host
 * models that must not allocate device memory at the point where they call
 * the chemistry: one that hands all free device memory to its own pool
 * allocator at start-up, or one whose time loop must not call cudaMalloc or
 * cudaFree because those calls synchronise the whole device and stall the
 * model's other streams.  Same semantics as mkpp_gpu_integrate_k in plain
 * mode (one thread per cell); the caller passes the inputs and outputs, and
 * the LU and stage scratch is a static device array inside the library,
 * sized for MKPP_NOALLOC_MAX_CELLS cells: 1024 x NSLOTS doubles (SAPRC99
 * 18.2 MB, saprcnov 17.3 MB, TS1 85.2 MB, saprc99_mini 1.2 MB; Chapman and
 * small_strato keep their store in registers and use none), which every GPU
 * that loads the library holds until the process exits.  Larger num_cells
 * is rejected with MKPP_ERROR_INVALID_ARGUMENT and a message on stderr.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current and keeps it for the
 * process; make that first call before any stream capture, and make no call
 * after a cudaDeviceReset of that device, which leaves the kept address
 * stale.  All calls share the array: calls that overlap on the GPU (other
 * streams, other host threads) race and must not be issued.  Nothing in the
 * array needs clearing between calls; each cell's slots are written before
 * they are read.  Makes no cudaMalloc or cudaFree call. */
#define MKPP_NOALLOC_MAX_CELLS 1024
int mkpp_gpu_integrate_noalloc(size_t num_cells, double* conc, const double* ktab,
                               size_t k_step_stride, int steps, double dt, double seed,
                               int max_attempts, int* status, int* accepted, int* rejected,
                               void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MKPP_GB300_MKPP_H */

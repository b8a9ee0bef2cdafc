// Driver of the reference's generated CPU solver (TEST AND CPU-BASELINE
// INFRASTRUCTURE ONLY).  Compiled by oracle/ref_build.py against the headers
// the MKPP compiler regenerated into oracle/_ref/gen/<mech>/ and the Kokkos
// shim.  For every cell it binds the state as a strided view of the
// LayoutLeft (cells x species) array and the cell's runtime parameter row,
// and calls the unmodified SolverKernels<D>::integrate() `steps` times, the
// per-cell body of ParamsTiledCellIntegrator
// (src/mkpp_host/include/mkpp_host/dispatcher.hpp:225-254), with the cells
// split over OpenMP threads in static chunks of 64 like the reference's
// RangePolicy(0, cells, ChunkSize(64)) (mechanism_manager.hpp:125-127).
#include <omp.h>

#include <vector>

#include MKPP_REF_HEADER

namespace {
struct HostDevice {
  using memory_space = Kokkos::HostSpace;
};
using Solver = MKPP_REF_NS::SolverKernels<HostDevice>;
using ParamView = Kokkos::View<const double*, Kokkos::HostSpace>;
using StateView = Kokkos::View<double*, Kokkos::LayoutStride, Kokkos::HostSpace>;

// One host step of one cell, with the environment arguments the mechanism's
// integrate() signature takes (integrate.j2: runtime environment and cloud
// gating add trailing arguments).  A template so that only the matching
// branch is instantiated.
template <class S>
void step(const S& solver, double dt, StateView& state, const ParamView& jvals, double t, double rh, double clw,
          double rho) {
  if constexpr (S::SUPPORTS_RUNTIME_ENVIRONMENT) {
    if constexpr (S::HAS_CLOUD_GATED) {
      solver.integrate(dt, state, jvals, t, rh, clw, rho);
    } else {
      solver.integrate(dt, state, jvals, t, rh, rho);
    }
  } else {
    solver.integrate(dt, state, jvals);
  }
}

template <class S, class V, class O>
void rates(const S& solver, const V& state, O& out, const ParamView& jvals, double t, double rh, double clw,
           double rho) {
  if constexpr (S::SUPPORTS_RUNTIME_ENVIRONMENT) {
    if constexpr (S::HAS_CLOUD_GATED) {
      solver.compute_rates(state, out, jvals, t, rh, clw, rho);
    } else {
      solver.compute_rates(state, out, jvals, t, rh, rho);
    }
  } else {
    solver.compute_rates(state, out, jvals);
  }
}

template <class S, class V, class O>
void jacobian(const S& solver, const V& state, O& out, const ParamView& jvals, double t, double rh, double clw,
              double rho) {
  if constexpr (S::SUPPORTS_RUNTIME_ENVIRONMENT) {
    if constexpr (S::HAS_CLOUD_GATED) {
      solver.compute_jacobian(state, out, jvals, t, rh, clw, rho);
    } else {
      solver.compute_jacobian(state, out, jvals, t, rh, rho);
    }
  } else {
    solver.compute_jacobian(state, out, jvals);
  }
}
}  // namespace

extern "C" {

int mkpp_ref_num_species() { return Solver::NUM_SPECIES; }
int mkpp_ref_num_parameters() { return Solver::NUM_RUNTIME_PARAMETERS; }

// conc[s * ncells + c] (in/out), param[p * ncells + c] with nparam rows; clw
// (cloud liquid water, cloud-gated mechanisms only) may be null for 0.
// chunk: cells per static OpenMP chunk, 64 as the reference's
// RangePolicy(0, cells, ChunkSize(64)); a smaller chunk keeps every thread
// busy on a sample of fewer than 64 cells per thread.
int mkpp_ref_integrate(int ncells, double* conc, const double* temp, const double* rh, const double* clw,
                       const double* rho, const double* param, int nparam, double dt, int steps, int nthreads,
                       double seed, int chunk) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  const int np = Solver::NUM_RUNTIME_PARAMETERS > 0 ? Solver::NUM_RUNTIME_PARAMETERS : 1;
  if (chunk < 1) chunk = 64;
#pragma omp parallel
  {
    std::vector<double> forcing(np, 0.0);
#pragma omp for schedule(static, chunk)
    for (int c = 0; c < ncells; ++c) {
      Solver solver;
      if (seed > 0.0) solver.initial_step_seed = seed;
      for (int p = 0; p < np; ++p) forcing[p] = p < nparam ? param[(size_t)p * ncells + c] : 0.0;
      ParamView jvals(forcing.data(), (std::size_t)np);
      StateView state(conc + c, Solver::NUM_SPECIES, (std::size_t)ncells);
      const double w = clw ? clw[c] : 0.0;
      for (int s = 0; s < steps; ++s) step(solver, dt, state, jvals, temp[c], rh[c], w, rho[c]);
    }
  }
  return 0;
}

// Tendencies F[s * ncells + c] from the reference's compute_rates().
int mkpp_ref_rates(int ncells, const double* conc, const double* temp, const double* rh, const double* clw,
                   const double* rho, const double* param, int nparam, double* out) {
  const int np = Solver::NUM_RUNTIME_PARAMETERS > 0 ? Solver::NUM_RUNTIME_PARAMETERS : 1;
  std::vector<double> forcing(np, 0.0);
  Solver solver;
  for (int c = 0; c < ncells; ++c) {
    for (int p = 0; p < np; ++p) forcing[p] = p < nparam ? param[(size_t)p * ncells + c] : 0.0;
    ParamView jvals(forcing.data(), (std::size_t)np);
    Kokkos::View<const double*, Kokkos::LayoutStride, Kokkos::HostSpace> state(conc + c, Solver::NUM_SPECIES,
                                                                               (std::size_t)ncells);
    StateView f(out + c, Solver::NUM_SPECIES, (std::size_t)ncells);
    for (int s = 0; s < Solver::NUM_SPECIES; ++s) f(s) = 0.0;
    rates(solver, state, f, jvals, temp[c], rh[c], clw ? clw[c] : 0.0, rho[c]);
  }
  return 0;
}

// Dense Jacobian J[(i * NS + j) * ncells + c] = dF_i/dC_j from compute_jacobian().
int mkpp_ref_jacobian(int ncells, const double* conc, const double* temp, const double* rh, const double* clw,
                      const double* rho, const double* param, int nparam, double* out) {
  const int np = Solver::NUM_RUNTIME_PARAMETERS > 0 ? Solver::NUM_RUNTIME_PARAMETERS : 1;
  const std::size_t ns = Solver::NUM_SPECIES;
  std::vector<double> forcing(np, 0.0);
  Solver solver;
  for (std::size_t e = 0; e < ns * ns * (std::size_t)ncells; ++e) out[e] = 0.0;
  for (int c = 0; c < ncells; ++c) {
    for (int p = 0; p < np; ++p) forcing[p] = p < nparam ? param[(size_t)p * ncells + c] : 0.0;
    ParamView jvals(forcing.data(), (std::size_t)np);
    Kokkos::View<const double*, Kokkos::LayoutStride, Kokkos::HostSpace> state(conc + c, ns, (std::size_t)ncells);
    Kokkos::View<double**, Kokkos::LayoutStride, Kokkos::HostSpace> jac(out + c, ns, ns, ns * ncells,
                                                                         (std::size_t)ncells);
    jacobian(solver, state, jac, jvals, temp[c], rh[c], clw ? clw[c] : 0.0, rho[c]);
  }
  return 0;
}

}  // extern "C"

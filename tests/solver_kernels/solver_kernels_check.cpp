// SolverKernels<DeviceType> (include/mkpp_gb300/solver_kernels.hpp) driven
// from a call site shaped like the reference's host dispatcher: a functor
// that, per cell, default-constructs the solver, gathers the cell's
// temperature, humidity, air density and forcing row, takes a rank-1 view of
// the cell's species in a LayoutLeft (cells x species) array and calls
// integrate() `steps` times with the signature the mechanism's constants
// select (src/mkpp_host/include/mkpp_host/dispatcher.hpp:101-122,225-254).
// Views are the host Kokkos stand-in of oracle/kokkos_shim (TEST ONLY).
//
//   solver_kernels_check <dir> <cells> <dt> <steps>
// reads <dir>/{conc,temp,rh,rho,param}.bin (float64, LayoutLeft, cell
// innermost) and writes
//   deferred.bin  integrate() with mkpp_gb300::Cuda (cells recorded under
//                 OpenMP, solved at the fence)
//   sync.bin      integrate() with mkpp_gb300::CudaSync (one cell per call)
//   registry.bin  mkpp::host::MechanismRegistry::execute on the same inputs
//   rates.bin, jacobian.bin, tlm.bin, adjoint.bin  compute_* of every cell
//                 at its input state (dense NS x NS for the matrices, zero
//                 outside the written pattern; tlm with delta = state)
//   status.bin    last_cell_status() of each cell after the deferred fence
// With no GPU the first solve throws std::runtime_error ("FATAL ERROR: ..."),
// which ends the program with status 3.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "Kokkos_Core.hpp"
#include MKPP_KERNELS_HEADER

namespace gen = MKPP_KERNELS_NS;
using StateCol = Kokkos::View<double*, Kokkos::LayoutStride, Kokkos::HostSpace>;
using ConstRow = Kokkos::View<const double*, Kokkos::HostSpace>;

namespace {

std::vector<double> load(const std::string& path, std::size_t n) {
  std::vector<double> v(n);
  std::ifstream f(path, std::ios::binary);
  if (!f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * sizeof(double))))
    throw std::runtime_error("cannot read " + path);
  return v;
}

void save(const std::string& path, const std::vector<double>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(double)));
}

// The fields of the reference's BasicHostExecutionParams a cell call reads.
struct CellParams {
  double dt;
  ConstRow jvals;
  double temp, rh, clw, air_density;
};

// One integrate() call in the form the mechanism's constants select.
template <class Solver, class Params, class Sub>
void integrate_one(Solver& solver, const Params& p, Sub sub) {
  if constexpr (requires { Solver::SUPPORTS_RUNTIME_ENVIRONMENT; }) {
    if constexpr (Solver::SUPPORTS_RUNTIME_ENVIRONMENT) {
      if constexpr (Solver::HAS_CLOUD_GATED) {
        solver.integrate(p.dt, sub, p.jvals, p.temp, p.rh, p.clw, p.air_density);
      } else {
        solver.integrate(p.dt, sub, p.jvals, p.temp, p.rh, p.air_density);
      }
    } else {
      solver.integrate(p.dt, sub, p.jvals);
    }
  } else {
    solver.integrate(p.dt, sub, p.jvals);
  }
}

// compute_* of one cell in the form the mechanism's constants select.
template <class Solver, class State, class Out, class Mat, class Row>
void evaluate_one(const Solver& solver, State& st, Out& F, Out& dF, Mat& J, Mat& JA, const Row& jv, double temp,
                  double rh, double rho) {
  if constexpr (Solver::SUPPORTS_RUNTIME_ENVIRONMENT) {
    if constexpr (Solver::HAS_CLOUD_GATED) {
      solver.compute_rates(st, F, jv, temp, rh, 0.0, rho);
      solver.compute_jacobian(st, J, jv, temp, rh, 0.0, rho);
      solver.compute_tlm(st, st, dF, jv, temp, rh, 0.0, rho);
      solver.compute_adjoint(st, JA, jv, temp, rh, 0.0, rho);
    } else {
      solver.compute_rates(st, F, jv, temp, rh, rho);
      solver.compute_jacobian(st, J, jv, temp, rh, rho);
      solver.compute_tlm(st, st, dF, jv, temp, rh, rho);
      solver.compute_adjoint(st, JA, jv, temp, rh, rho);
    }
  } else {
    solver.compute_rates(st, F, jv);
    solver.compute_jacobian(st, J, jv);
    solver.compute_tlm(st, st, dF, jv);
    solver.compute_adjoint(st, JA, jv);
  }
}

template <class Device>
std::vector<double> run_cells(const std::vector<double>& conc0, const std::vector<double>& temp,
                              const std::vector<double>& rh, const std::vector<double>& rho,
                              const std::vector<double>& param, int n, double dt, int steps) {
  using Solver = gen::SolverKernels<Device>;
  const int ns = Solver::NUM_SPECIES;
  const int np = Solver::NUM_RUNTIME_PARAMETERS > 0 ? Solver::NUM_RUNTIME_PARAMETERS : 1;
  std::vector<double> work(conc0);
#pragma omp parallel for schedule(static, 64) if (Device::deferred)
  for (int c = 0; c < n; ++c) {
    Solver solver;
    std::vector<double> forcing(np, 0.0);
    for (int p = 0; p < Solver::NUM_RUNTIME_PARAMETERS; ++p) forcing[p] = param[(std::size_t)p * n + c];
    const CellParams params{dt, ConstRow(forcing.data(), (std::size_t)np), temp[c], rh[c], 0.0, rho[c]};
    StateCol sub(work.data() + c, (std::size_t)ns, (std::size_t)n);
    for (int s = 0; s < steps; ++s) integrate_one(solver, params, sub);
  }
  Device::fence();
  return work;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: %s <dir> <cells> <dt> <steps>\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  const int n = std::atoi(argv[2]);
  const double dt = std::atof(argv[3]);
  const int steps = std::atoi(argv[4]);
  using Solver = gen::SolverKernels<mkpp_gb300::Cuda>;
  const int ns = Solver::NUM_SPECIES;
  const int np = Solver::NUM_RUNTIME_PARAMETERS;
  static_assert(Solver::NUM_SPECIES == MKPP_NUM_SPECIES_CHECK, "species count");
  try {
    const auto conc0 = load(dir + "/conc.bin", (std::size_t)ns * n);
    const auto temp = load(dir + "/temp.bin", n);
    const auto rh = load(dir + "/rh.bin", n);
    const auto rho = load(dir + "/rho.bin", n);
    const auto param = load(dir + "/param.bin", (std::size_t)(np > 0 ? np : 1) * n);

    const auto deferred = run_cells<mkpp_gb300::Cuda>(conc0, temp, rh, rho, param, n, dt, steps);
    std::vector<double> status(n);
    for (int c = 0; c < n; ++c) status[c] = mkpp_gb300::last_cell_status(deferred.data() + c);
    save(dir + "/deferred.bin", deferred);
    save(dir + "/status.bin", status);
    save(dir + "/sync.bin", run_cells<mkpp_gb300::CudaSync>(conc0, temp, rh, rho, param, n, dt, steps));

    std::vector<double> reg(conc0);
    mkpp::host::HostExecutionParams hp;
    hp.dt = dt;
    hp.steps = steps;
    hp.cell_temperature = {temp.data(), (std::size_t)n, 1};
    hp.cell_humidity = {rh.data(), (std::size_t)n, 1};
    hp.cell_density = {rho.data(), (std::size_t)n, 1};
    if (np > 0) hp.cell_jvals = {param.data(), (std::size_t)n, (std::size_t)np, 1, n};
    mkpp::host::MechanismRegistry::execute(Solver::NAME, reg.data(), (std::size_t)n, hp);
    save(dir + "/registry.bin", reg);

    // compute_* at each cell's input state.
    std::vector<double> rates((std::size_t)ns * n), jac((std::size_t)ns * ns * n, 0.0), tlm((std::size_t)ns * n),
        adj((std::size_t)ns * ns * n, 0.0);
    std::vector<double> state(conc0);
    const Solver solver;
    for (int c = 0; c < n; ++c) {
      std::vector<double> forcing(np > 0 ? np : 1, 0.0);
      for (int p = 0; p < np; ++p) forcing[p] = param[(std::size_t)p * n + c];
      ConstRow jv(forcing.data(), forcing.size());
      StateCol st(state.data() + c, (std::size_t)ns, (std::size_t)n);
      StateCol F(rates.data() + c, (std::size_t)ns, (std::size_t)n);
      StateCol dF(tlm.data() + c, (std::size_t)ns, (std::size_t)n);
      // J(i, j) at jac[c + n * (i + ns * j)]
      Kokkos::View<double**, Kokkos::LayoutStride, Kokkos::HostSpace> J(jac.data() + c, ns, ns, (std::size_t)n,
                                                                       (std::size_t)n * ns);
      Kokkos::View<double**, Kokkos::LayoutStride, Kokkos::HostSpace> JA(adj.data() + c, ns, ns, (std::size_t)n,
                                                                        (std::size_t)n * ns);
      evaluate_one(solver, st, F, dF, J, JA, jv, temp[c], rh[c], rho[c]);
    }
    save(dir + "/rates.bin", rates);
    save(dir + "/jacobian.bin", jac);
    save(dir + "/tlm.bin", tlm);
    save(dir + "/adjoint.bin", adj);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 3;
  }
  return 0;
}

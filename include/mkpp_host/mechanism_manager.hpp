// mkpp_host/mechanism_manager.hpp - the reference's host dispatcher interface
// over the GB300 mechanism libraries (libmkpp_<mechanism>.so).
//
// Replaces, with the same names, argument meaning and error behaviour:
//   mkpp::host::MechanismRegistry::{get_registered_mechanisms, has_mechanism,
//     get_info, execute}   src/mkpp_host/include/mkpp_host/mechanism_manager.hpp:21-228
//   mkpp::host::BasicHostExecutionParams / HostExecutionParams
//                           src/mkpp_host/include/mkpp_host/dispatcher.hpp:79-97
//   mkpp::host::CellErrorCode   dispatcher.hpp:15-21
//   mkpp::host::BatchErrorStatus   dispatcher.hpp:124-144
//   the per-cell gather of ParamsTiledCellIntegrator   dispatcher.hpp:196-254
//   mkpp::host::execute_mechanism_steps[_batched], execute_mechanism
//                           dispatcher.hpp:319-384
//
// Differences, all forced by the absence of Kokkos on this side:
// * Views become pointers with extents (CellValues, CellForcing) and the state
//   is a LayoutLeft (cells x species) host array, state[cell + cells * species],
//   as the C ABI takes it.
// * Mechanisms are the libraries found in the library directory (environment
//   MKPP_GB300_LIB_DIR, else the MKPP_GB300_LIB_DIR macro, else
//   mkpp_gb300/lib), not the headers present at compile time.  Each library is
//   opened privately (RTLD_LOCAL): the C-ABI symbols are not
//   mechanism-namespaced.
// * execute() runs on the GPU through mkpp_integrate and can hand back the
//   per-cell status codes (CellErrorCode values).
// * get_info() reports the mechanism's reaction count (the reference leaves
//   it 0).  requires_env is false for every library built here: it is true in
//   the reference only for its equilibrium mechanism, which is not built.
// * The batched status holds every per-cell outcome of the solve (attempt cap,
//   numerical failure), not only the non-finite inputs the reference records;
//   team_size is accepted and unused (the GPU kernels size their own grids).
//
// Header-only, C++17; link with -ldl.  With the CUDA toolkit's include
// directory on the path, the batched dispatch opens the reference's NVTX
// range MKPP_Batched_Team_Dispatch_<name>.
#pragma once

#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <filesystem>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "mkpp.h"

// NVTX3 is header-only and ships with the CUDA toolkit; with its include
// directory on the path the batched dispatch opens an NVTX range, otherwise
// the range is a no-op.
#if defined(__has_include)
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define MKPP_HOST_NVTX 1
#endif
#endif

namespace mkpp {
namespace host {

// A named profiler range over a scope, as the reference's Kokkos profiling
// regions (Kokkos::Profiling::ScopedRegion).  Without a profiler attached,
// NVTX calls do nothing.
class TraceRange {
 public:
  explicit TraceRange(const std::string& name) {
#ifdef MKPP_HOST_NVTX
    nvtxRangePushA(name.c_str());
#else
    (void)name;
#endif
  }
  ~TraceRange() {
#ifdef MKPP_HOST_NVTX
    nvtxRangePop();
#endif
  }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

enum CellErrorCode : int {
  SUCCESS = MKPP_CELL_SUCCESS,
  ERR_SINGULAR_MATRIX = MKPP_CELL_ERR_SINGULAR_MATRIX,
  ERR_NON_FINITE_STATE = MKPP_CELL_ERR_NON_FINITE_STATE,
  ERR_CONVERGENCE_FAILURE = MKPP_CELL_ERR_CONVERGENCE,
  ERR_NUMERICAL_FAILURE = MKPP_CELL_ERR_NUMERICAL
};

template <typename MemorySpace = void>
struct BatchErrorStatus {
  std::vector<int> status;

  BatchErrorStatus() = default;
  explicit BatchErrorStatus(std::size_t num_cells) : status(num_cells, SUCCESS) {}
  void set_error(std::size_t cell_idx, CellErrorCode code) { status[cell_idx] = static_cast<int>(code); }
  int get_error(std::size_t cell_idx) const { return status[cell_idx]; }
};

struct MechanismInfo {
  std::string name;
  int num_species{0};
  int num_reactions{0};
  bool requires_env{false};
};

// One value per cell: data[cell * stride], extent cells (0: not supplied).
struct CellValues {
  const double* data{nullptr};
  std::size_t extent{0};
  std::ptrdiff_t stride{1};
  double operator()(std::size_t cell) const { return data[static_cast<std::ptrdiff_t>(cell) * stride]; }
};

// Runtime parameter rows per cell: data[cell * cell_stride + slot * slot_stride]
// (the reference's LayoutStride cell_jvals view; cells 0: not supplied).
struct CellForcing {
  const double* data{nullptr};
  std::size_t cells{0};
  std::size_t slots{0};
  std::ptrdiff_t cell_stride{1};
  std::ptrdiff_t slot_stride{0};
  double operator()(std::size_t cell, std::size_t slot) const {
    return data[static_cast<std::ptrdiff_t>(cell) * cell_stride + static_cast<std::ptrdiff_t>(slot) * slot_stride];
  }
};

struct HostExecutionParams {
  double dt{60.0};                  // seconds per integrate() call
  const double* jvals{nullptr};     // one parameter row shared by every cell (null: zeros)
  std::size_t jvals_count{0};       // entries of jvals
  double temp{288.15};              // K, for cells without cell_temperature
  double air_density{2.4476e19};
  CellValues cell_temperature;
  CellValues cell_humidity;
  CellValues cell_density;
  CellValues cell_cloud_water;
  CellForcing cell_jvals;
  double rh{0.5};
  double clw{0.0};
  int steps{1};                     // integrate() calls per cell
  std::size_t jvals_extent{512};    // kept for source compatibility; zeros need no buffer here
};

namespace detail {

struct Library {
  std::string name;
  void* so{nullptr};
  int num_species{0}, num_variable{0}, num_reactions{0}, num_parameters{0}, num_lu{0};
  int (*sizes)(int*, int*, int*, int*, int*){nullptr};
  int (*create)(mkpp_handle_t*, size_t){nullptr};
  int (*initialize)(mkpp_handle_t){nullptr};
  int (*set_state)(mkpp_handle_t, double*, const double*, const double*, const double*){nullptr};
  int (*set_params)(mkpp_handle_t, const double*, size_t){nullptr};
  int (*set_cloud)(mkpp_handle_t, const double*){nullptr};
  int (*set_aerosol)(mkpp_handle_t, const double*, const double*){nullptr};
  int (*integrate)(mkpp_handle_t, double){nullptr};
  int (*cell_stats)(mkpp_handle_t, int*, int*, int*){nullptr};
  int (*last_error)(mkpp_handle_t, char*, size_t){nullptr};
  int (*set_seed)(mkpp_handle_t, double){nullptr};
  int (*evaluate_rates)(mkpp_handle_t, double*){nullptr};
  int (*evaluate_jacobian)(mkpp_handle_t, double*){nullptr};
  int (*jacobian_vector)(mkpp_handle_t, const double*, double*){nullptr};
  int (*jacobian_transpose_vector)(mkpp_handle_t, const double*, double*){nullptr};
  std::map<std::size_t, mkpp_handle_t> handles;  // one per cell count, kept for the process
  // Handles of the per-cell SolverKernels entry points
  // (mkpp_gb300/solver_kernels.hpp), kept apart because those set the seed.
  std::map<std::size_t, mkpp_handle_t> kernel_handles;
};

inline std::string library_dir() {
  if (const char* env = std::getenv("MKPP_GB300_LIB_DIR")) return env;
#ifdef MKPP_GB300_LIB_DIR
  return MKPP_GB300_LIB_DIR;
#else
  return "mkpp_gb300/lib";
#endif
}

inline std::vector<std::string> scan() {
  std::vector<std::string> names;
  std::error_code ec;
  for (const auto& e : std::filesystem::directory_iterator(library_dir(), ec)) {
    const std::string f = e.path().filename().string();
    const std::string pre = "libmkpp_", suf = ".so";
    if (f.size() > pre.size() + suf.size() && f.compare(0, pre.size(), pre) == 0 &&
        f.compare(f.size() - suf.size(), suf.size(), suf) == 0)
      names.push_back(f.substr(pre.size(), f.size() - pre.size() - suf.size()));
  }
  std::sort(names.begin(), names.end());
  return names;
}

[[noreturn]] inline void unknown(const std::string& name) {
  std::string err = "FATAL ERROR: Unknown mechanism '" + name + "'. Supported: ";
  const auto list = scan();
  for (std::size_t i = 0; i < list.size(); ++i) err += list[i] + (i + 1 < list.size() ? ", " : "");
  std::cerr << err << std::endl;
  throw std::runtime_error(err);
}

template <class F>
void bind(Library& lib, F& fn, const char* symbol) {
  fn = reinterpret_cast<F>(dlsym(lib.so, symbol));
  if (!fn) throw std::runtime_error("FATAL ERROR: " + lib.name + " library lacks " + symbol);
}

inline std::mutex& lock() {
  static std::mutex m;
  return m;
}

// Opened libraries stay loaded (and their handles allocated) until the
// process exits; nothing is torn down from static destructors, after which
// the CUDA runtime may already be gone.
inline Library& library(const std::string& name) {
  static auto* libs = new std::map<std::string, Library*>();
  auto it = libs->find(name);
  if (it != libs->end()) return *it->second;
  const auto list = scan();
  if (std::find(list.begin(), list.end(), name) == list.end()) unknown(name);
  const std::string path = library_dir() + "/libmkpp_" + name + ".so";
  void* so = dlopen(path.c_str(), RTLD_NOW | RTLD_LOCAL);
  if (!so) throw std::runtime_error("FATAL ERROR: cannot load " + path + ": " + dlerror());
  auto* lib = new Library();
  lib->name = name;
  lib->so = so;
  bind(*lib, lib->sizes, "mkpp_mechanism_sizes");
  bind(*lib, lib->create, "mkpp_create_handle");
  bind(*lib, lib->initialize, "mkpp_initialize");
  bind(*lib, lib->set_state, "mkpp_set_state_ptrs");
  bind(*lib, lib->set_params, "mkpp_set_rate_parameter_ptrs");
  bind(*lib, lib->set_cloud, "mkpp_set_cloud_water_ptr");
  bind(*lib, lib->set_aerosol, "mkpp_set_aerosol_ptrs");
  bind(*lib, lib->integrate, "mkpp_integrate");
  bind(*lib, lib->cell_stats, "mkpp_get_cell_stats");
  bind(*lib, lib->last_error, "mkpp_get_last_error");
  bind(*lib, lib->set_seed, "mkpp_set_initial_step_seed");
  bind(*lib, lib->evaluate_rates, "mkpp_evaluate_rates");
  bind(*lib, lib->evaluate_jacobian, "mkpp_evaluate_jacobian");
  bind(*lib, lib->jacobian_vector, "mkpp_evaluate_jacobian_vector");
  bind(*lib, lib->jacobian_transpose_vector, "mkpp_evaluate_jacobian_transpose_vector");
  lib->sizes(&lib->num_species, &lib->num_variable, &lib->num_reactions, &lib->num_parameters, &lib->num_lu);
  (*libs)[name] = lib;
  return *lib;
}

[[noreturn]] inline void fail(Library& lib, mkpp_handle_t h, int rc, const char* what) {
  char msg[512] = {0};
  if (h) lib.last_error(h, msg, sizeof msg);
  std::string err = msg[0] ? std::string(msg)
                           : "FATAL ERROR: " + std::string(what) + " returned " + std::to_string(rc) + " for " + lib.name;
  std::cerr << err << std::endl;
  throw std::runtime_error(err);
}

// The library's handle for n cells from `pool` (lib.handles unless given),
// created and initialised on first use (call with lock() held).
inline mkpp_handle_t handle(Library& lib, std::size_t n, std::map<std::size_t, mkpp_handle_t>* pool = nullptr) {
  mkpp_handle_t& h = (pool ? *pool : lib.handles)[n];
  if (!h) {
    int rc = lib.create(&h, n);
    if (rc != MKPP_SUCCESS) {
      h = nullptr;
      fail(lib, nullptr, rc, "mkpp_create_handle");
    }
    rc = lib.initialize(h);
    if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_initialize");
  }
  return h;
}

}  // namespace detail

class MechanismRegistry {
 public:
  static std::vector<std::string> get_registered_mechanisms() { return detail::scan(); }

  static bool has_mechanism(const std::string& name) {
    const auto list = get_registered_mechanisms();
    return std::find(list.begin(), list.end(), name) != list.end();
  }

  static MechanismInfo get_info(const std::string& name) {
    std::lock_guard<std::mutex> g(detail::lock());
    detail::Library& lib = detail::library(name);
    return {name, lib.num_species, lib.num_reactions, false};
  }

  // Integrates every cell of `state` (LayoutLeft cells x species, in place)
  // `params.steps` times over params.dt, with the reference's per-cell
  // gather: per-cell meteorology and forcing where supplied, the scalars and
  // the shared parameter row otherwise.  Per-cell outcomes go to cell_status
  // (num_cells CellErrorCode values) when it is not null.
  static void execute(const std::string& name, double* state, std::size_t num_cells,
                      const HostExecutionParams& params, int* cell_status = nullptr) {
    std::lock_guard<std::mutex> g(detail::lock());
    detail::Library& lib = detail::library(name);
    for (const std::size_t extent : {params.cell_temperature.extent, params.cell_humidity.extent,
                                     params.cell_density.extent, params.cell_cloud_water.extent}) {
      if (extent != 0 && extent != num_cells)
        throw std::invalid_argument("FATAL ERROR: per-cell meteorology extent does not match state");
    }
    if (params.cell_jvals.cells != 0 && params.cell_jvals.cells != num_cells)
      throw std::invalid_argument("FATAL ERROR: per-cell forcing extent does not match state");
    if (params.cell_jvals.cells != 0 && params.cell_jvals.slots < static_cast<std::size_t>(lib.num_parameters))
      throw std::invalid_argument("FATAL ERROR: per-cell forcing has too few runtime parameters");
    if (num_cells == 0) return;
    if (!state) throw std::invalid_argument("FATAL ERROR: state pointer is null");

    const std::size_t n = num_cells;
    const std::size_t np = static_cast<std::size_t>(lib.num_parameters);
    std::vector<double> temp(n), rho(n), rh(n), clw(n), pressure(n, 101325.0), forcing(n * std::max<std::size_t>(np, 1));
    for (std::size_t c = 0; c < n; ++c) {
      temp[c] = params.cell_temperature.extent ? params.cell_temperature(c) : params.temp;
      rho[c] = params.cell_density.extent ? params.cell_density(c) : params.air_density;
      rh[c] = params.cell_humidity.extent ? params.cell_humidity(c) : params.rh;
      clw[c] = params.cell_cloud_water.extent ? params.cell_cloud_water(c) : params.clw;
      for (std::size_t p = 0; p < np; ++p) {
        double v = 0.0;
        if (params.cell_jvals.cells) v = params.cell_jvals(c, p);
        else if (params.jvals && p < params.jvals_count) v = params.jvals[p];
        forcing[c + n * p] = v;
      }
    }

    mkpp_handle_t h = detail::handle(lib, n);
    int rc = lib.set_state(h, state, temp.data(), pressure.data(), rho.data());
    if (rc != MKPP_SUCCESS) detail::fail(lib, h, rc, "mkpp_set_state_ptrs");
    rc = lib.set_aerosol(h, rh.data(), nullptr);
    if (rc != MKPP_SUCCESS) detail::fail(lib, h, rc, "mkpp_set_aerosol_ptrs");
    rc = lib.set_cloud(h, clw.data());
    if (rc != MKPP_SUCCESS) detail::fail(lib, h, rc, "mkpp_set_cloud_water_ptr");
    if (np > 0) {
      rc = lib.set_params(h, forcing.data(), np);
      if (rc != MKPP_SUCCESS) detail::fail(lib, h, rc, "mkpp_set_rate_parameter_ptrs");
    }
    std::vector<int> status(n, SUCCESS), step_status(n);
    for (int s = 0; s < params.steps; ++s) {
      rc = lib.integrate(h, params.dt);
      if (rc != MKPP_SUCCESS) detail::fail(lib, h, rc, "mkpp_integrate");
      rc = lib.cell_stats(h, step_status.data(), nullptr, nullptr);
      if (rc != MKPP_SUCCESS) detail::fail(lib, h, rc, "mkpp_get_cell_stats");
      for (std::size_t c = 0; c < n; ++c)
        if (status[c] == SUCCESS) status[c] = step_status[c];
    }
    if (cell_status) std::copy(status.begin(), status.end(), cell_status);
  }
};

// `steps` integrate() calls of dt on every cell, with one parameter row
// shared by all cells (null: zeros).
inline void execute_mechanism_steps(const std::string& name, double* state, std::size_t num_cells, double dt,
                                    int steps, const double* jvals = nullptr, std::size_t jvals_count = 0) {
  HostExecutionParams p;
  p.dt = dt;
  p.steps = steps;
  p.jvals = jvals;
  p.jvals_count = jvals_count;
  MechanismRegistry::execute(name, state, num_cells, p);
}

inline void execute_mechanism(const std::string& name, double* state, std::size_t num_cells, double dt,
                              const double* jvals = nullptr, std::size_t jvals_count = 0) {
  execute_mechanism_steps(name, state, num_cells, dt, 1, jvals, jvals_count);
}

// As execute_mechanism_steps, with fault isolation: a cell with a non-finite
// input is left untouched and flagged ERR_NON_FINITE_STATE, every other cell
// integrates, and one summary line goes to stderr when any cell faulted.
template <typename MemorySpace>
void execute_mechanism_steps_batched(const std::string& name, double* state, std::size_t num_cells, double dt,
                                     int steps, const double* jvals, std::size_t jvals_count,
                                     BatchErrorStatus<MemorySpace>& error_status, int team_size = 64) {
  (void)team_size;
  if (error_status.status.size() < num_cells) {
    std::string err = "FATAL ERROR: batched integration error buffer (" + std::to_string(error_status.status.size()) +
                      ") smaller than batch (" + std::to_string(num_cells) + ").";
    std::cerr << err << std::endl;
    throw std::runtime_error(err);
  }
  // The reference's region name (dispatcher.hpp:335).
  const TraceRange range("MKPP_Batched_Team_Dispatch_" + name);
  HostExecutionParams p;
  p.dt = dt;
  p.steps = steps;
  p.jvals = jvals;
  p.jvals_count = jvals_count;
  MechanismRegistry::execute(name, state, num_cells, p, error_status.status.data());
  std::size_t faulted = 0;
  for (std::size_t c = 0; c < num_cells; ++c) faulted += error_status.status[c] != SUCCESS;
  if (faulted > 0) {
    std::cerr << "FATAL ERROR: batched integration of '" << name << "' reported " << faulted << " faulted cell(s) of "
              << num_cells << "; per-cell codes are in the status buffer\n";
  }
}

}  // namespace host
}  // namespace mkpp

// mkpp_gb300/solver_kernels.hpp - the reference's generated C++ solver API,
// SolverKernels<DeviceType>, over the GB300 mechanism libraries.
//
// Replaces, with the same names, signatures and meaning:
//   template <class DeviceType> struct SolverKernels   src/mkpp/templates/header.j2:127-132
//   NUM_SPECIES, NUM_RUNTIME_PARAMETERS, NUM_PHOTOLYSIS,
//   SUPPORTS_RUNTIME_ENVIRONMENT, HAS_CLOUD_GATED, atol[], rtol[]
//                                                      header.j2:128-131,185-203
//   double initial_step_seed                           solver_variants/integrate.j2:34-42
//   integrate(dt_total, state, jvals[, temp, rh[, clw], air_density])
//                                                      solver_variants/integrate.j2:52-67
//   compute_rates(state, F, jvals[, env])              kernel_functions/compute_rates.j2:16-42
//   compute_jacobian(state, J, jvals[, env])           kernel_functions/compute_jacobian.j2:16-45
//   compute_tlm(state, delta, dF, jvals[, env]),
//   compute_adjoint(state, J_adj, jvals[, env])        kernel_functions/compute_{tlm,adjoint}.j2
//                                                      (under MKPP_ENABLE_ADJOINT, as there)
// The per-mechanism header generated/host_api/<m>/<m>.hpp supplies the
// constants and the Species enum in namespace mkpp::generated::<m>, as the
// reference's generated <m>.hpp does, and names this template SolverKernels.
//
// Views.  Any Kokkos-like view works: the state needs operator()(i) returning
// a reference (a rank-1 subview of a cells x species array, for instance),
// jvals needs data() and extent(0).  Missing trailing environment arguments
// take the reference's defaults (the compile-time temperature and air
// density, rh 0.5, clw 0).  jvals shorter than NUM_RUNTIME_PARAMETERS is
// padded with zeros.
//
// Execution.  The reference calls integrate() once per cell inside a Kokkos
// parallel_for on its device type.  Here the device type decides when the
// cell reaches the GPU:
//   mkpp_gb300::Cuda      integrate() records the cell (state address,
//                         forcing, environment, dt, seed) and returns;
//                         mkpp_gb300::fence() (also Cuda::fence()) solves
//                         every recorded cell in batched mkpp_integrate calls
//                         and writes each state back.  As with a Kokkos
//                         device space, results are visible after the fence.
//                         Repeated calls on one state run in call order.
//   mkpp_gb300::CudaSync  integrate() solves its one cell before returning.
// Both give each cell exactly the result of the batched C ABI on the same
// inputs: the per-cell arithmetic does not depend on the batch.  compute_*
// evaluate on the GPU before they return, for either device type.  Recording
// is thread safe (the reference's call sites run under OpenMP); a fence
// solves what every thread recorded.
//
// Errors: a failing C ABI call throws std::runtime_error with the library's
// "FATAL ERROR:" message.  A cell that fails numerically ends with the state
// the solver left (the reference's integrate() has no status either); the
// status of the cells of the last fence is available from last_cell_status().
//
// The reference's integrate_fwd_checkpoint / integrate_adj / integrate_tlm
// (a frozen-Jacobian reverse sweep over at most 200 steps) have no member
// here: the libraries' differentiation is the discrete adjoint and tangent
// of mkpp_gpu_integrate_checkpoint / mkpp_gpu_adjoint / mkpp_gpu_tangent.
//
// Header-only, C++17; link with -ldl.  The libraries are found as the host
// registry finds them (MKPP_GB300_LIB_DIR).
#pragma once

#include <algorithm>
#include <cstddef>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../mkpp_host/mechanism_manager.hpp"

namespace mkpp_gb300 {

// Memory the views live in: host memory of the caller.
struct HostMemory {
  using memory_space = HostMemory;
};

namespace sk_detail {

// One recorded integrate() call.
struct Call {
  double dt, seed, temp, rh, clw, rho;
  std::vector<double> forcing;
};

// One recorded state: where its species live and its calls in order.
struct Cell {
  double* base;
  std::ptrdiff_t stride;
  std::vector<Call> calls;
};

struct Queue {
  std::vector<Cell> cells;
  std::unordered_map<double*, std::size_t> index;
};

inline std::mutex& queue_lock() {
  static std::mutex m;
  return m;
}

inline std::map<std::string, Queue>& queues() {
  static auto* q = new std::map<std::string, Queue>();
  return *q;
}

// Per-cell status of the last fence, by state address.
inline std::unordered_map<const double*, int>& last_status() {
  static auto* s = new std::unordered_map<const double*, int>();
  return *s;
}

// Solves the recorded cells of one mechanism: round r runs the r-th call of
// every cell that has one, one mkpp_integrate per (dt, seed) group.  Call
// with no lock held.
inline void solve(const std::string& name, std::vector<Cell>& cells) {
  using mkpp::host::detail::fail;
  std::lock_guard<std::mutex> g(mkpp::host::detail::lock());
  mkpp::host::detail::Library& lib = mkpp::host::detail::library(name);
  const std::size_t ns = static_cast<std::size_t>(lib.num_species);
  const std::size_t np = static_cast<std::size_t>(lib.num_parameters);
  std::size_t rounds = 0;
  for (const Cell& c : cells) rounds = std::max(rounds, c.calls.size());
  for (std::size_t r = 0; r < rounds; ++r) {
    std::map<std::pair<double, double>, std::vector<std::size_t>> groups;
    for (std::size_t i = 0; i < cells.size(); ++i)
      if (cells[i].calls.size() > r) groups[{cells[i].calls[r].dt, cells[i].calls[r].seed}].push_back(i);
    for (const auto& grp : groups) {
      const std::vector<std::size_t>& ids = grp.second;
      const std::size_t n = ids.size();
      std::vector<double> conc(n * ns), temp(n), pressure(n, 101325.0), rho(n), rh(n), clw(n),
          forcing(n * std::max<std::size_t>(np, 1), 0.0);
      for (std::size_t k = 0; k < n; ++k) {
        const Cell& c = cells[ids[k]];
        const Call& call = c.calls[r];
        for (std::size_t s = 0; s < ns; ++s) conc[k + n * s] = c.base[static_cast<std::ptrdiff_t>(s) * c.stride];
        temp[k] = call.temp;
        rho[k] = call.rho;
        rh[k] = call.rh;
        clw[k] = call.clw;
        for (std::size_t p = 0; p < np && p < call.forcing.size(); ++p) forcing[k + n * p] = call.forcing[p];
      }
      mkpp_handle_t h = mkpp::host::detail::handle(lib, n, &lib.kernel_handles);
      int rc = lib.set_seed(h, grp.first.second);
      if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_set_initial_step_seed");
      rc = lib.set_state(h, conc.data(), temp.data(), pressure.data(), rho.data());
      if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_set_state_ptrs");
      rc = lib.set_aerosol(h, rh.data(), nullptr);
      if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_set_aerosol_ptrs");
      rc = lib.set_cloud(h, clw.data());
      if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_set_cloud_water_ptr");
      if (np > 0) {
        rc = lib.set_params(h, forcing.data(), np);
        if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_set_rate_parameter_ptrs");
      }
      rc = lib.integrate(h, grp.first.first);
      if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_integrate");
      std::vector<int> status(n);
      rc = lib.cell_stats(h, status.data(), nullptr, nullptr);
      if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_get_cell_stats");
      for (std::size_t k = 0; k < n; ++k) {
        const Cell& c = cells[ids[k]];
        for (std::size_t s = 0; s < ns; ++s) c.base[static_cast<std::ptrdiff_t>(s) * c.stride] = conc[k + n * s];
        int& st = last_status()[c.base];
        if (r == 0 || st == MKPP_CELL_SUCCESS) st = status[k];
      }
    }
  }
}

// Solves every mechanism's recorded cells.
inline void fence_all() {
  std::map<std::string, Queue> work;
  {
    std::lock_guard<std::mutex> g(queue_lock());
    work.swap(queues());
  }
  {
    std::lock_guard<std::mutex> g(mkpp::host::detail::lock());
    last_status().clear();
  }
  for (auto& q : work) solve(q.first, q.second.cells);
}

template <class V>
std::size_t extent0(const V& v) {
  return static_cast<std::size_t>(v.extent(0));
}

template <class... T>
struct all_arithmetic : std::true_type {};
template <class H, class... T>
struct all_arithmetic<H, T...>
    : std::integral_constant<bool, std::is_arithmetic<H>::value && all_arithmetic<T...>::value> {};

}  // namespace sk_detail

// Solves every cell recorded by SolverKernels<mkpp_gb300::Cuda>::integrate().
inline void fence() { sk_detail::fence_all(); }

// Status (MKPP_CELL_* code) of the cell whose state starts at `state` in
// the last fence or synchronous integrate(); MKPP_CELL_SUCCESS when unknown.
inline int last_cell_status(const double* state) {
  std::lock_guard<std::mutex> g(mkpp::host::detail::lock());
  auto it = sk_detail::last_status().find(state);
  return it == sk_detail::last_status().end() ? MKPP_CELL_SUCCESS : it->second;
}

// Deferred device type: cells are solved at the next fence.
struct Cuda {
  using memory_space = HostMemory;
  using execution_space = Cuda;
  static constexpr bool deferred = true;
  static void fence() { ::mkpp_gb300::fence(); }
};

// Synchronous device type: each integrate() solves its cell before it returns.
struct CudaSync {
  using memory_space = HostMemory;
  using execution_space = CudaSync;
  static constexpr bool deferred = false;
  static void fence() {}
};

// The per-mechanism SolverKernels derive from this; C holds the mechanism's
// constants (NAME, NUM_SPECIES, ..., atol, rtol, the Jacobian pattern).
template <class C, class DeviceType>
struct SolverKernelsBase : C {
  using memory_space = typename DeviceType::memory_space;

  // Trailing environment arguments integrate() and compute_* take after
  // jvals: none without a runtime environment, else temp, rh[, clw],
  // air_density.
  static constexpr std::size_t kEnvArgs = C::SUPPORTS_RUNTIME_ENVIRONMENT ? (C::HAS_CLOUD_GATED ? 4 : 3) : 0;

  // First substep of every integrate() is dt_total * initial_step_seed.
  double initial_step_seed = C::INITIAL_STEP_SEED;

  template <class StateView, class JView, class... Env,
            typename std::enable_if<(sizeof...(Env) <= kEnvArgs) && sk_detail::all_arithmetic<Env...>::value,
                                    int>::type = 0>
  void integrate(double dt_total, StateView& state, const JView& jvals, Env... env) const {
    sk_detail::Call call = make_call(dt_total, jvals, env...);
    double* base = &state(0);
    const std::ptrdiff_t stride = &state(1) - &state(0);
    {
      std::lock_guard<std::mutex> g(sk_detail::queue_lock());
      sk_detail::Queue& q = sk_detail::queues()[C::NAME];
      auto it = q.index.find(base);
      if (it == q.index.end()) {
        q.index.emplace(base, q.cells.size());
        q.cells.push_back(sk_detail::Cell{base, stride, {}});
        it = q.index.find(base);
      }
      q.cells[it->second].calls.push_back(std::move(call));
    }
    if (!DeviceType::deferred) ::mkpp_gb300::fence();
  }

  template <class StateView, class RateView, class JView, class... Env,
            typename std::enable_if<(sizeof...(Env) <= kEnvArgs) && sk_detail::all_arithmetic<Env...>::value,
                                    int>::type = 0>
  void compute_rates(const StateView& state, RateView& F, const JView& jvals, Env... env) const {
    std::vector<double> out(C::NUM_SPECIES);
    evaluate(state, make_call(0.0, jvals, env...), [&](mkpp::host::detail::Library& lib, mkpp_handle_t h) {
      return lib.evaluate_rates(h, out.data());
    });
    for (int i = 0; i < C::NUM_SPECIES; ++i) F(i) = out[i];
  }

  // J(i, j) = dF_i / dC_j at the reference's sparse pattern; other entries
  // are left as they are.
  template <class StateView, class JacView, class JView, class... Env,
            typename std::enable_if<(sizeof...(Env) <= kEnvArgs) && sk_detail::all_arithmetic<Env...>::value,
                                    int>::type = 0>
  void compute_jacobian(const StateView& state, JacView& J, const JView& jvals, Env... env) const {
    const std::vector<double> d = dense_jacobian(state, make_call(0.0, jvals, env...));
    for (int e = 0; e < C::NUM_JACOBIAN_ENTRIES; ++e) {
      const int i = C::jacobian_pattern[e][0], j = C::jacobian_pattern[e][1];
      J(i, j) = d[i + C::NUM_SPECIES * j];
    }
  }

#ifdef MKPP_ENABLE_ADJOINT
  // J_adj(i, j) = J(j, i) at the transposed pattern.
  template <class StateView, class JacView, class JView, class... Env,
            typename std::enable_if<(sizeof...(Env) <= kEnvArgs) && sk_detail::all_arithmetic<Env...>::value,
                                    int>::type = 0>
  void compute_adjoint(const StateView& state, JacView& J_adj, const JView& jvals, Env... env) const {
    const std::vector<double> d = dense_jacobian(state, make_call(0.0, jvals, env...));
    for (int e = 0; e < C::NUM_JACOBIAN_ENTRIES; ++e) {
      const int i = C::jacobian_pattern[e][0], j = C::jacobian_pattern[e][1];
      J_adj(j, i) = d[i + C::NUM_SPECIES * j];
    }
  }

  // dF = J delta_C.
  template <class StateView, class DeltaView, class RateView, class JView, class... Env,
            typename std::enable_if<(sizeof...(Env) <= kEnvArgs) && sk_detail::all_arithmetic<Env...>::value,
                                    int>::type = 0>
  void compute_tlm(const StateView& state, const DeltaView& delta_C, RateView& dF, const JView& jvals,
                   Env... env) const {
    std::vector<double> delta(C::NUM_SPECIES), out(C::NUM_SPECIES);
    for (int i = 0; i < C::NUM_SPECIES; ++i) delta[i] = delta_C(i);
    evaluate(state, make_call(0.0, jvals, env...), [&](mkpp::host::detail::Library& lib, mkpp_handle_t h) {
      return lib.jacobian_vector(h, delta.data(), out.data());
    });
    for (int i = 0; i < C::NUM_SPECIES; ++i) dF(i) = out[i];
  }
#endif

 private:
  template <class JView, class... Env>
  sk_detail::Call make_call(double dt, const JView& jvals, Env... env) const {
    double e[4] = {C::ENV_TEMPERATURE, 0.5, 0.0, C::ENV_AIR_DENSITY};  // temp, rh, clw, air_density
    const double given[sizeof...(Env) + 1] = {static_cast<double>(env)..., 0.0};
    // Positional: temp, rh, [clw,] air_density.
    const int slot[4] = {0, 1, C::HAS_CLOUD_GATED ? 2 : 3, 3};
    for (std::size_t a = 0; a < sizeof...(Env); ++a) e[slot[a]] = given[a];
    sk_detail::Call call{dt, initial_step_seed, e[0], e[1], e[2], e[3], {}};
    const std::size_t np = C::NUM_RUNTIME_PARAMETERS;
    call.forcing.assign(np, 0.0);
    const double* p = jvals.data();
    const std::size_t have = p ? std::min(np, sk_detail::extent0(jvals)) : 0;
    for (std::size_t i = 0; i < have; ++i) call.forcing[i] = p[i];
    return call;
  }

  // One cell through a 1-cell handle, then `run` (an evaluation entry).
  template <class StateView, class Run>
  void evaluate(const StateView& state, const sk_detail::Call& call, Run&& run) const {
    using mkpp::host::detail::fail;
    std::lock_guard<std::mutex> g(mkpp::host::detail::lock());
    mkpp::host::detail::Library& lib = mkpp::host::detail::library(C::NAME);
    std::vector<double> conc(C::NUM_SPECIES);
    for (int i = 0; i < C::NUM_SPECIES; ++i) conc[i] = state(i);
    double temp = call.temp, pressure = 101325.0, rho = call.rho, rh = call.rh, clw = call.clw;
    mkpp_handle_t h = mkpp::host::detail::handle(lib, 1, &lib.kernel_handles);
    int rc = lib.set_state(h, conc.data(), &temp, &pressure, &rho);
    if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_set_state_ptrs");
    rc = lib.set_aerosol(h, &rh, nullptr);
    if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_set_aerosol_ptrs");
    rc = lib.set_cloud(h, &clw);
    if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_set_cloud_water_ptr");
    if (C::NUM_RUNTIME_PARAMETERS > 0) {
      rc = lib.set_params(h, call.forcing.data(), call.forcing.size());
      if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_set_rate_parameter_ptrs");
    }
    rc = run(lib, h);
    if (rc != MKPP_SUCCESS) fail(lib, h, rc, "mkpp_evaluate");
  }

  template <class StateView>
  std::vector<double> dense_jacobian(const StateView& state, const sk_detail::Call& call) const {
    std::vector<double> d(static_cast<std::size_t>(C::NUM_SPECIES) * C::NUM_SPECIES);
    evaluate(state, call, [&](mkpp::host::detail::Library& lib, mkpp_handle_t h) {
      return lib.evaluate_jacobian(h, d.data());
    });
    return d;
  }
};

}  // namespace mkpp_gb300

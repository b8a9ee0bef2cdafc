// Drives include/mkpp_host/mechanism_manager.hpp for tests/test_registry.py
// (TEST INFRASTRUCTURE ONLY).
//   registry_check list                  registered mechanisms, one per line
//   registry_check info <m>              "<name> <species> <reactions> <requires_env>"
//   registry_check unknown <m>           get_info on a name that is not registered
//   registry_check extent <m>            execute with a mismatched per-cell extent
//   registry_check forcing <m>           execute with too few forcing slots
//   registry_check execute <m> <n> <dt> <steps> <dir>
//       reads <dir>/{conc,temp,rho,rh,param}.bin (float64, LayoutLeft), runs
//       execute(), writes <dir>/{conc_out,status}.bin
//   registry_check batched <m> <n> <dt> <steps> <dir>
//       reads <dir>/{conc,jvals}.bin, runs execute_mechanism_steps_batched()
//       with the shared parameter row, writes <dir>/{conc_out,status}.bin
// The error modes print the exception's message and exit 3 when it is the
// expected kind, 1 otherwise.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "mkpp_host/mechanism_manager.hpp"

using mkpp::host::MechanismRegistry;

static std::vector<double> read(const std::string& path, size_t count) {
  std::vector<double> v(count);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(count * sizeof(double)));
  if (!f) throw std::runtime_error("short read: " + path);
  return v;
}

template <class T>
static void write(const std::string& path, const std::vector<T>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string mode = argv[1];
  const std::string mech = argc > 2 ? argv[2] : "";
  if (mode == "list") {
    for (const auto& m : MechanismRegistry::get_registered_mechanisms())
      std::cout << m << (MechanismRegistry::has_mechanism(m) ? "" : " (not found)") << "\n";
    return MechanismRegistry::has_mechanism("no_such_mechanism") ? 1 : 0;
  }
  if (mode == "info") {
    const auto i = MechanismRegistry::get_info(mech);
    std::cout << i.name << " " << i.num_species << " " << i.num_reactions << " " << int(i.requires_env) << "\n";
    return 0;
  }
  if (mode == "unknown") {
    try {
      MechanismRegistry::get_info(mech);
    } catch (const std::runtime_error& e) {
      std::cout << e.what() << "\n";
      return 3;
    }
    return 1;
  }
  if (mode == "extent" || mode == "forcing") {
    const size_t n = 8;
    const auto info = MechanismRegistry::get_info(mech);
    std::vector<double> conc(n * info.num_species, 1.0), t(n - 1, 300.0), row(n, 0.0);
    mkpp::host::HostExecutionParams p;
    if (mode == "extent") {
      p.cell_temperature = {t.data(), t.size(), 1};
    } else {
      p.cell_jvals = {row.data(), n, 1, 1, 0};
    }
    try {
      MechanismRegistry::execute(mech, conc.data(), n, p);
    } catch (const std::invalid_argument& e) {
      std::cout << e.what() << "\n";
      return 3;
    }
    return 1;
  }
  if (mode == "execute" && argc == 7) {
    const size_t n = std::stoul(argv[3]);
    const double dt = std::stod(argv[4]);
    const int steps = std::stoi(argv[5]);
    const std::string dir = argv[6];
    const auto info = MechanismRegistry::get_info(mech);
    size_t np = 0;
    {
      std::ifstream f(dir + "/param.bin", std::ios::binary | std::ios::ate);
      np = static_cast<size_t>(f.tellg()) / sizeof(double) / n;
    }
    auto conc = read(dir + "/conc.bin", n * info.num_species);
    auto temp = read(dir + "/temp.bin", n), rho = read(dir + "/rho.bin", n), rh = read(dir + "/rh.bin", n);
    auto param = np ? read(dir + "/param.bin", n * np) : std::vector<double>();
    mkpp::host::HostExecutionParams p;
    p.dt = dt;
    p.steps = steps;
    p.cell_temperature = {temp.data(), n, 1};
    p.cell_density = {rho.data(), n, 1};
    p.cell_humidity = {rh.data(), n, 1};
    if (np) p.cell_jvals = {param.data(), n, np, 1, static_cast<std::ptrdiff_t>(n)};
    std::vector<int> status(n);
    MechanismRegistry::execute(mech, conc.data(), n, p, status.data());
    write(dir + "/conc_out.bin", conc);
    write(dir + "/status.bin", status);
    return 0;
  }
  if (mode == "batched" && argc == 7) {
    const size_t n = std::stoul(argv[3]);
    const double dt = std::stod(argv[4]);
    const int steps = std::stoi(argv[5]);
    const std::string dir = argv[6];
    const auto info = MechanismRegistry::get_info(mech);
    size_t np = 0;
    {
      std::ifstream f(dir + "/jvals.bin", std::ios::binary | std::ios::ate);
      np = static_cast<size_t>(f.tellg()) / sizeof(double);
    }
    auto conc = read(dir + "/conc.bin", n * info.num_species);
    auto jvals = np ? read(dir + "/jvals.bin", np) : std::vector<double>();
    mkpp::host::BatchErrorStatus<> err(n);
    mkpp::host::execute_mechanism_steps_batched(mech, conc.data(), n, dt, steps, jvals.data(), np, err);
    write(dir + "/conc_out.bin", conc);
    write(dir + "/status.bin", err.status);
    return 0;
  }
  return 2;
}

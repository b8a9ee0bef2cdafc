// small_strato_rodas3.hpp of the small_strato_rodas3 library (libmkpp_small_strato_rodas3.so), generated from its
// plan: the reference's generated C++ solver API for this mechanism
// (src/mkpp/templates/header.j2:70-80,127-203), namespace
// mkpp::generated::small_strato_rodas3 with enum Species and SolverKernels<DeviceType>.
// The members and their execution are described in
// include/mkpp_gb300/solver_kernels.hpp.
#pragma once

#include "../../../../include/mkpp_gb300/solver_kernels.hpp"

namespace mkpp {
namespace generated {
namespace small_strato_rodas3 {

enum Species : int {
    O = 0,
    O1D = 1,
    O3 = 2,
    NO = 3,
    NO2 = 4,
    M = 5,
    O2 = 6
};

struct MechanismConstants {
  static constexpr const char* NAME = "small_strato_rodas3";
  static constexpr int NUM_SPECIES = 7;
  static constexpr int NUM_RUNTIME_PARAMETERS = 4;
  static constexpr int NUM_PHOTOLYSIS = 4;
  static constexpr int NUM_REACTIONS = 10;
  static constexpr bool SUPPORTS_RUNTIME_ENVIRONMENT = false;
  static constexpr bool HAS_CLOUD_GATED = false;
  static constexpr double ENV_TEMPERATURE = 298.15;
  static constexpr double ENV_AIR_DENSITY = 2.46e+19;
  static constexpr double INITIAL_STEP_SEED = 1e-06;
  static constexpr double atol[NUM_SPECIES] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0};
  static constexpr double rtol[NUM_SPECIES] = {0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001};
  // (row, column) of the Jacobian entries compute_jacobian writes
  static constexpr int NUM_JACOBIAN_ENTRIES = 28;
  static constexpr int jacobian_pattern[NUM_JACOBIAN_ENTRIES][2] = {{0, 0}, {0, 1}, {0, 2}, {0, 4}, {0, 5}, {0, 6}, {1, 1}, {1, 2}, {1, 5}, {2, 0}, {2, 1}, {2, 2}, {2, 3}, {2, 6}, {3, 0}, {3, 2}, {3, 3}, {3, 4}, {4, 0}, {4, 2}, {4, 3}, {4, 4}, {6, 0}, {6, 1}, {6, 2}, {6, 3}, {6, 4}, {6, 6}};
};

template <class DeviceType>
struct SolverKernels : ::mkpp_gb300::SolverKernelsBase<MechanismConstants, DeviceType> {};

}  // namespace small_strato_rodas3
}  // namespace generated
}  // namespace mkpp

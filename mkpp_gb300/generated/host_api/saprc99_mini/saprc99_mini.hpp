// saprc99_mini.hpp of the saprc99_mini library (libmkpp_saprc99_mini.so), generated from its
// plan: the reference's generated C++ solver API for this mechanism
// (src/mkpp/templates/header.j2:70-80,127-203), namespace
// mkpp::generated::saprc99_mini with enum Species and SolverKernels<DeviceType>.
// The members and their execution are described in
// include/mkpp_gb300/solver_kernels.hpp.
#pragma once

#include "../../../../include/mkpp_gb300/solver_kernels.hpp"

namespace mkpp {
namespace generated {
namespace saprc99_mini {

enum Species : int {
    O3 = 0,
    H2O2 = 1,
    NO = 2,
    NO2 = 3,
    NO3 = 4,
    N2O5 = 5,
    HONO = 6,
    HNO3 = 7,
    HNO4 = 8,
    O3P = 9,
    OH = 10,
    HO2 = 11,
    AIR = 12,
    O2 = 13,
    H2O = 14,
    M = 15,
    N2 = 16
};

struct MechanismConstants {
  static constexpr const char* NAME = "saprc99_mini";
  static constexpr int NUM_SPECIES = 17;
  static constexpr int NUM_RUNTIME_PARAMETERS = 4;
  static constexpr int NUM_PHOTOLYSIS = 4;
  static constexpr int NUM_REACTIONS = 13;
  static constexpr bool SUPPORTS_RUNTIME_ENVIRONMENT = true;
  static constexpr bool HAS_CLOUD_GATED = false;
  static constexpr double ENV_TEMPERATURE = 298.15;
  static constexpr double ENV_AIR_DENSITY = 2.46e+19;
  static constexpr double INITIAL_STEP_SEED = 1e-06;
  static constexpr double atol[NUM_SPECIES] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0};
  static constexpr double rtol[NUM_SPECIES] = {0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001};
  // (row, column) of the Jacobian entries compute_jacobian writes
  static constexpr int NUM_JACOBIAN_ENTRIES = 54;
  static constexpr int jacobian_pattern[NUM_JACOBIAN_ENTRIES][2] = {{0, 0}, {0, 2}, {0, 3}, {0, 9}, {0, 12}, {0, 13}, {1, 1}, {1, 11}, {1, 12}, {2, 0}, {2, 2}, {2, 3}, {2, 4}, {2, 6}, {3, 0}, {3, 2}, {3, 3}, {3, 4}, {3, 5}, {3, 7}, {3, 12}, {4, 0}, {4, 2}, {4, 3}, {4, 4}, {4, 5}, {4, 7}, {4, 10}, {4, 12}, {5, 3}, {5, 4}, {5, 5}, {5, 12}, {6, 6}, {7, 7}, {7, 10}, {7, 12}, {9, 0}, {9, 3}, {9, 9}, {9, 12}, {9, 13}, {10, 1}, {10, 6}, {10, 7}, {10, 10}, {10, 12}, {11, 11}, {11, 12}, {13, 0}, {13, 9}, {13, 11}, {13, 12}, {13, 13}};
};

template <class DeviceType>
struct SolverKernels : ::mkpp_gb300::SolverKernelsBase<MechanismConstants, DeviceType> {};

}  // namespace saprc99_mini
}  // namespace generated
}  // namespace mkpp

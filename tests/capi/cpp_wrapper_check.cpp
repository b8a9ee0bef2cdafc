// Drives the reference's generated C++ wrapper (mkpp.hpp, produced at test
// time by the reference compiler) against this repository's mkpp.h and a
// mechanism library (TEST INFRASTRUCTURE ONLY; run by
// tests/test_capi_contract.py).  No call here computes.  Prints "ok".
#include <cstdio>
#include <stdexcept>
#include <vector>

#include "mkpp.hpp"

int main() {
  const std::size_t n = 8;
  mkpp::MechanismContext ctx(n);
  ctx.initialize();
  if (ctx.getSpeciesCount() != MKPP_NUM_SPECIES || ctx.getReactionCount() != MKPP_NUM_REACTIONS ||
      ctx.getPhotolysisCount() != MKPP_NUM_PHOTOLYSIS)
    return 1;
  if (ctx.getSpeciesIndex("O3") < 0) return 2;
  std::vector<double> conc(n * MKPP_NUM_SPECIES, 1e9), t(n, 298.15), p(n, 101325.0), rho(n, 2.45e19);
  std::vector<double> prm(n * (MKPP_NUM_RATE_PARAMETERS > 0 ? MKPP_NUM_RATE_PARAMETERS : 1), 0.0);
  ctx.setStatePointers(conc.data(), t.data(), p.data(), rho.data());
  ctx.setRateParameterPointers(prm.data(), MKPP_NUM_RATE_PARAMETERS);
  try {
    ctx.integrate(0.0);  // invalid dt: the wrapper turns the C status into an exception
    return 3;
  } catch (const std::exception&) {
  }
  std::puts("ok");
  return 0;
}

// One Rosenbrock attempt of an emitted mechanism header, on the host (TEST
// INFRASTRUCTURE ONLY).  The store is a plain array of the per-cell slots
// (the layout of Mech: Y, stage vectors K0.., F, DY, KT), the rate constants
// a plain array.
#include MKPP_MECH_HEADER

namespace {
using Mech = MKPP_MECH_NS::Mech;

struct Store {
  double* p;
  double& operator[](int s) const { return p[s]; }
};

struct Rates {
  const double* k;
  double operator()(int r) const { return k[r]; }
};
}  // namespace

extern "C" {

// NSLOTS, NV, NR, NSTAGE, Y, K0, F, DY, KT
int hostsim_layout(int* out) {
  const int v[9] = {Mech::NSLOTS, Mech::NV, Mech::NR, Mech::NSTAGE, Mech::Y, Mech::K0, Mech::F, Mech::DY, Mech::KT};
  for (int i = 0; i < 9; ++i) out[i] = v[i];
  return 0;
}

double hostsim_attempt(double* slots, const double* k, double h, int* status) {
  Store S{slots};
  int st = 0;
  const double err = Mech::attempt(S, Rates{k}, h, st);
  *status = st;
  return err;
}

}  // extern "C"

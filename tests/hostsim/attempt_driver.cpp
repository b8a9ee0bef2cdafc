// The rate constants, one Rosenbrock attempt, and the adjoint and tangent of
// one step, of an emitted mechanism header on the host (TEST INFRASTRUCTURE
// ONLY).  The store is a plain array of the per-cell slots (the layout of
// Mech: Y, stage vectors K0.., F, DY, KT), the rate constants a plain array.
#include <vector>

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

struct Row {
  const double* v;
  double operator()(int i) const { return v ? v[i] : 0.0; }
};

struct RowOut {
  double* v;
  void set(int i, double x) const { v[i] = x; }
};

// Tendencies F[s] and the dense Jacobian J[row + NS * col] of one cell from
// the emitted fun(), jac_w() (with 1/(gamma h) = 0, negated) and
// jac_fixed_columns(), composed as the evaluation kernels compose them; for
// a table-driven mechanism from eval_step() on a slot store instead of the
// first two.
template <class M>
int evaluate(const double* conc, const double* param, double T, double RHO, double RH, double CLW,
             const double* k, double* F, double* J) {
  if constexpr (M::TABLE_ATTEMPT) {
    const int NS = M::NS;
    std::vector<double> slots(M::NSLOTS, 0.0);
    Store S{slots.data()};
    for (int i = 0; i < M::NV; ++i) S[M::Y + i] = conc[M::var_phys(i)];
    M::eval_step(S, Rates{k});
    for (int s = 0; s < NS; ++s) F[s] = 0.0;
    for (int e = 0; e < NS * NS; ++e) J[e] = 0.0;
    for (int i = 0; i < M::NV; ++i) F[M::var_phys(i)] = S[M::F + i];
    M::for_each_w_slot([&](int slot, int, int) { J[M::lu_prow(slot) + NS * M::lu_pcol(slot)] = -S[slot]; });
    struct Y {
      const double* c;
      double operator()(int i) const { return c[M::var_phys(i)]; }
    } y{conc};
    M::jac_fixed_columns(Row{param}, Row{conc}, T, RHO, RH, CLW, y,
                         [&](int row, int col, double v) { J[row + NS * col] = v; });
    return 0;
  } else {
    const int NS = M::NS;
    struct Y {
      const double* c;
      double operator()(int i) const { return c[M::var_phys(i)]; }
    } y{conc};
    struct Dense {
      double* J;
      double& operator[](int s) const { return J[M::lu_prow(s) + M::NS * M::lu_pcol(s)]; }
    } S{J};
    for (int s = 0; s < NS; ++s) F[s] = 0.0;
    for (int e = 0; e < NS * NS; ++e) J[e] = 0.0;
    M::fun(y, Rates{k}, [&](int i, double v) { F[M::var_phys(i)] = v; });
    M::jac_w(y, Rates{k}, 0.0, S);
    M::for_each_w_slot([&](int slot, int, int) { S[slot] = -S[slot]; });
    M::jac_fixed_columns(Row{param}, Row{conc}, T, RHO, RH, CLW, y,
                         [&](int row, int col, double v) { J[row + NS * col] = v; });
    return 0;
  }
}
}  // namespace

extern "C" {

// Rate constants of one cell from the emitted rate_constants(): conc holds
// the cell's NS concentrations (the fixed species are read), param its
// runtime parameters (null: zeros); k receives NR values.
void hostsim_rate_constants(const double* conc, const double* param, double T, double RHO, double RH, double CLW,
                            double* k) {
  RowOut out{k};
  Mech::rate_constants(Row{param}, Row{conc}, T, RHO, RH, CLW, out);
}

// Tendencies and dense Jacobian of one cell (evaluate() above).
int hostsim_evaluate(const double* conc, const double* param, double T, double RHO, double RH, double CLW,
                     const double* k, double* F, double* J) {
  return evaluate<Mech>(conc, param, T, RHO, RH, CLW, k, F, J);
}

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

// LAM, KB, NSLOTS_ADJ
int hostsim_adj_layout(int* out) {
  out[0] = Mech::LAM;
  out[1] = Mech::KB;
  out[2] = Mech::NSLOTS_ADJ;
  return 0;
}

// The reverse of one step of size h, as the adjoint kernel runs it: the step
// recomputed with attempt(), then adjoint_step() (lambda in S[LAM..] in,
// dL/dy_n out; dL/dk added to S[KB..]).
void hostsim_adjoint(double* slots, const double* k, double h, int* status) {
  Store S{slots};
  int st = 0;
  Mech::attempt(S, Rates{k}, h, st);
  Mech::adjoint_step(S, Rates{k}, h);
  *status = st;
}

// DYT, DKR, NSLOTS_TLM
int hostsim_tlm_layout(int* out) {
  out[0] = Mech::DYT;
  out[1] = Mech::DKR;
  out[2] = Mech::NSLOTS_TLM;
  return 0;
}

// The tangent of one step of size h: attempt(), then tlm_step() (dy in
// S[DYT..] and dk in S[DKR..] in, dy_new in S[DYT..] out).
void hostsim_tlm(double* slots, const double* k, double h, int* status) {
  Store S{slots};
  int st = 0;
  Mech::attempt(S, Rates{k}, h, st);
  Mech::tlm_step(S, Rates{k}, h);
  *status = st;
}

}  // extern "C"

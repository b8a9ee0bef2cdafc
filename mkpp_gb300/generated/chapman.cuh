// Generated by mkpp_gb300.emitter.cuda_emitter from mechanisms/chapman.plan.json.
// Do not edit: regenerate with `python -m mkpp_gb300.emitter.cuda_emitter`.
// 4 species (3 variable), 4 reactions, 9 W slots, 9 LU slots, 5 LU products, 3 pivot scalings.
#pragma once
#include "mkpp_device.cuh"
namespace mkpp_chapman {

// Tables of the warp-cooperative attempt (device constant data).
namespace coop {
static __device__ const int r_off[5] = {0, 1, 3, 4, 6};
static __device__ const int r_y[6] = {2, 1, 2, 0, 1, 0};
static __device__ const int f_off[4] = {0, 3, 7, 11};
static __device__ const int f_r[11] = {1, 2, 3, 0, 1, 2, 3, 0, 1, 2, 3};
static __device__ const double f_c[11] = {1.0, -1.0, -1.0, 2.0, -1.0, 1.0, -1.0, -1.0, -1.0, 1.0, 2.0};
static __device__ const int d_r[6] = {0, 1, 1, 2, 3, 3};
static __device__ const int d_off[7] = {0, 0, 1, 2, 2, 3, 4};
static __device__ const int d_fac[4] = {2, 1, 0, 1};
static __device__ const double d_lit[6] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0};
static __device__ const int w_slot[9] = {0, 1, 2, 3, 4, 5, 6, 7, 8};
static __device__ const int w_diag[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
static __device__ const int w_off[10] = {0, 2, 4, 5, 7, 9, 11, 13, 15, 17};
static __device__ const int w_p[17] = {3, 5, 1, 4, 2, 3, 5, 1, 4, 0, 2, 3, 5, 1, 4, 0, 2};
static __device__ const double w_c[17] = {1.0, 1.0, -1.0, 1.0, -1.0, -1.0, 1.0, 1.0, 1.0, -2.0, 1.0, -1.0, -2.0, 1.0, -2.0, 1.0, 1.0};
constexpr int NW = 9;
constexpr int N_LU_ZERO = 0;
static __device__ const int lu_zero[1] = {0};
constexpr int LU_STEPS = 7;
constexpr int SV_STEPS = 8;
static __device__ const unsigned long long lu_fs[224] = {
    0x3000000000000ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2000000000003ull, 0x2000000000006ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000100030004ull, 0x1000200030005ull, 0x1000100060007ull, 0x1000200060008ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x3000000000004ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2000400000007ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000500070008ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x3000000000008ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
};
static __device__ const unsigned long long sv_fs[256] = {
    0x1000000030001ull, 0x1000000060002ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000100070002ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2000800000002ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000200050001ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2000400000001ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000100010000ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000200020000ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2000000000000ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
};
static __device__ const int diag[3] = {0, 4, 8};
}  // namespace coop


struct Mech {
  static constexpr const char* NAME = "chapman";
  static constexpr int NS = 4;      // species including fixed ones
  static constexpr int NV = 3;      // variable species (solved system)
  static constexpr int NR = 4;      // reactions
  static constexpr int NP = 2;      // runtime parameter slots per cell
  static constexpr int NPH = 2;      // photolysis slots
  static constexpr int NFIX = 1;
  static constexpr int NLU = 9;
  static constexpr int NSTAGE = 3;
  static constexpr bool RUNTIME_ENV = false;
  static constexpr bool CLOUD_GATED = false;
  static constexpr double GAMMA = 0.435866521508459;
  static constexpr double ELO = 3.0;
  static constexpr double SEED = 9.9999999999999995e-07;
  static constexpr double ENV_T = 298.14999999999998;
  static constexpr double ENV_RHO = 2.46e+19;
  static constexpr long long LU_FMA = 5;
  static constexpr long long LU_SCALE = 3;
  static constexpr long long SOLVE_L = 3;
  static constexpr long long SOLVE_U = 3;
  static constexpr long long FUN_FLOPS = 28;
  static constexpr long long JAC_FLOPS = 38;

  __host__ __device__ static constexpr int var_phys(int i) { constexpr int t[3] = {2, 0, 1}; return t[i]; }
  __host__ __device__ static constexpr int fix_phys(int i) { constexpr int t[1] = {3}; return t[i]; }
  __host__ __device__ static constexpr double atol_v(int i) { constexpr double t[3] = {1.0, 1.0, 1.0}; return t[i]; }
  __host__ __device__ static constexpr double rtol_v(int i) { constexpr double t[3] = {0.001, 0.001, 0.001}; return t[i]; }
  __host__ __device__ static constexpr int lu_prow(int s) { constexpr int t[9] = {2, 2, 2, 0, 0, 0, 1, 1, 1}; return t[s]; }
  __host__ __device__ static constexpr int lu_pcol(int s) { constexpr int t[9] = {2, 0, 1, 2, 0, 1, 2, 0, 1}; return t[s]; }
  static const char* species_name(int s) { static const char* t[4] = {"O", "O2", "O3", "M"}; return t[s]; }
  static const char* photolysis_name(int p) { static const char* t[2] = {"J_1", "J_2"}; return t[p]; }

  // Rate constants of every reaction (reaction index order).  P(n) is the
  // cell's runtime parameter n (photolysis J_n or external Rate slot n),
  // FIX(s) the concentration of fixed species s, T/RHO the cell's
  // temperature and air density.
  template <class PA, class FA, class KO>
  __device__ __forceinline__ static void rate_constants(const PA& P, const FA& FIX, double T, double RHO,
                                                      double RH, double CLW, KO& k) {
    (void)T; (void)RHO; (void)RH; (void)CLW; (void)P; (void)FIX;
    k.set(0, P(0));
    k.set(1, 6.0e-34*FIX(3));
    k.set(2, P(1));
    k.set(3, 7.9999999999999998e-12);
  }

  // Per-cell working storage, in slots of one double: the LU factors, the
  // state y, the stage vectors K_1..K_s, the tendency F, the increment dy and
  // the rate constants of the current host step.
  static constexpr int Y = 9;
  static constexpr int K0 = 12;
  static constexpr int F = 21;
  static constexpr int DY = 24;
  static constexpr int KT = 27;        // the cell's rate constants for the current host step
  static constexpr int NSLOTS = 31;

  // Mass-action tendencies F(y) of the variable species (logical order):
  // y(i) supplies the state, out(i, F_i) receives the result.
  template <class YA, class KA, class FO>
  __device__ __forceinline__ static void fun(const YA& y, const KA& k, FO&& out) {
    const double y0 = y(0);
    const double y1 = y(1);
    const double y2 = y(2);
    const double q0 = k(0) * y2;
    const double q1 = k(1) * y1 * y2;
    const double q2 = k(2) * y0;
    const double q3 = k(3) * y1 * y0;
    out(0, q1 - q2 - q3);
    out(1, 2.0 * q0 - q1 + q2 - q3);
    out(2, fma(2.0, q3, -q0 - q1 + q2));
  }

  // W = I/(gamma h) - J(y) into the LU slots that hold W entries.
  template <class YA, class KA, class SA>
  __device__ __forceinline__ static void jac_w(const YA& y, const KA& k, double inv_g_dt, SA& S) {
    (void)inv_g_dt;
    const double y0 = y(0);
    const double y1 = y(1);
    const double y2 = y(2);
    const double d0_2 = k(0);
    const double d1_1 = k(1) * y2;
    const double d1_2 = k(1) * y1;
    const double d2_0 = k(2);
    const double d3_1 = k(3) * y0;
    const double d3_0 = k(3) * y1;
    S[0] = inv_g_dt + d2_0 + d3_0;
    S[1] = -d1_1 + d3_1;
    S[2] = -d1_2;
    S[3] = -d2_0 + d3_0;
    S[4] = inv_g_dt + d1_1 + d3_1;
    S[5] = -2.0 * d0_2 + d1_2;
    S[6] = fma(-2.0, d3_0, -d2_0);
    S[7] = fma(-2.0, d3_1, d1_1);
    S[8] = inv_g_dt + d0_2 + d1_2;
  }

  // Physical (row, column) of every W slot, for the dense Jacobian.
  template <class Fn>
  __device__ __forceinline__ static void for_each_w_slot(Fn&& fn) {
    fn(0, 2, 2);
    fn(1, 2, 0);
    fn(2, 2, 1);
    fn(3, 0, 2);
    fn(4, 0, 0);
    fn(5, 0, 1);
    fn(6, 1, 2);
    fn(7, 1, 0);
    fn(8, 1, 1);
  }

  // Fixed-species columns of the dense Jacobian: dF_i/dC_f through the
  // rate constants' dependence on fixed species (third bodies).
  template <class PA, class FA, class YA, class Fn>
  __device__ __forceinline__ static void jac_fixed_columns(const PA& P, const FA& FIX, double T, double RHO,
                                                         double RH, double CLW, const YA& y, Fn&& fn) {
    (void)T; (void)RHO; (void)RH; (void)CLW; (void)P; (void)FIX; (void)y;
    fn(0, 3, -((6.0e-34) * y(1) * y(2)));
    fn(1, 3, -((6.0e-34) * y(1) * y(2)));
    fn(2, 3, ((6.0e-34) * y(1) * y(2)));
  }

  // In-place row-wise Doolittle LU over the compact slots, in the operation
  // order of the reference plan.  The operands a row reuses (its own L
  // entries for the U part, the pivot column of U for the L part) are read
  // once into registers.  Diagonal slots end up holding 1/U_ii.
  template <class SA>
  __device__ __forceinline__ static bool factor(SA& S) {
    bool ok = true;
    {  // pivot row 0
      const double u0 = S[0];
      ok = ok && (u0 != 0.0);
      const double rd = 1.0 / u0;
      S[0] = rd;
      double v1 = S[1];
      double v2 = S[2];
      double v3 = S[3];
      double v6 = S[6];
      S[3] = v3 * rd;
      S[6] = v6 * rd;
    }
    {  // pivot row 1
      const double a3 = S[3];
      const double u4 = fma(-a3, S[1], S[4]);
      ok = ok && (u4 != 0.0);
      const double rd = 1.0 / u4;
      S[4] = rd;
      double v5 = S[5];
      v5 = fma(-a3, S[2], v5);
      S[5] = v5;
      const double b1 = S[1];
      double v7 = S[7];
      v7 = fma(-S[6], b1, v7);
      S[7] = v7 * rd;
    }
    {  // pivot row 2
      const double a6 = S[6];
      const double a7 = S[7];
      const double u8 = fma(-a7, S[5], fma(-a6, S[2], S[8]));
      ok = ok && (u8 != 0.0);
      const double rd = 1.0 / u8;
      S[8] = rd;
    }
    return ok;
  }

  // Solve (LU) x = b in place on slots [base, base + NV): unit-L forward
  // sweep, then the U backward sweep scaled by the stored 1/U_ii.
  template <class SA>
  __device__ __forceinline__ static void solve(SA& S, const int base) {
    const double v0 = S[base + 0];
    const double v1 = fma(-S[3], v0, S[base + 1]);
    const double v2 = fma(-S[7], v1, fma(-S[6], v0, S[base + 2]));
    const double x2 = (v2) * S[8];
    S[base + 2] = x2;
    const double x1 = (fma(-S[5], x2, v1)) * S[4];
    S[base + 1] = x1;
    const double x0 = (fma(-S[2], x2, fma(-S[1], x1, v0))) * S[0];
    S[base + 0] = x0;
  }

  // One Rosenbrock attempt of size h from the state in S[Y..].  Returns the
  // WRMS error norm and leaves the increment sum_j M_j K_j in S[DY..].
  // Bit 1 of status is set on a zero pivot.
  template <class SA, class KA>
  __device__ __forceinline__ static double attempt(SA& S, const KA& k, double h, int& status) {
    const double inv_g_dt = 1.0 / (GAMMA * h);
    jac_w([&](int i) { return S[Y + i]; }, k, inv_g_dt, S);
    if (!factor(S)) status |= 1;
    fun([&](int i) { return S[Y + i]; }, k, [&](int i, double v) { S[F + i] = v; });
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[12 + i] = S[F + i];
    }
    solve(S, 12);
    fun([&](int i) { return S[Y + i] + S[12 + i]; }, k, [&](int i, double v) { S[F + i] = v; });
    const double c21 = -1.0156171083877703 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[15 + i] = fma(c21, S[12 + i], S[F + i]);
    }
    solve(S, 15);
    const double c31 = 4.0759956452537702 / h;
    const double c32 = 9.20767942983308 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[18 + i] = fma(c32, S[15 + i], fma(c31, S[12 + i], S[F + i]));
    }
    solve(S, 18);
    double err_sq = 0.0;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      const double k0 = S[12 + i];
      const double k1 = S[15 + i];
      const double k2 = S[18 + i];
      const double yi = S[Y + i];
      const double ynew = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, yi + k0));
      S[DY + i] = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, k0));
      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));
      const double q = (fma(0.22354069897811571, k2, fma(-2.9079558716805471, k1, 0.5 * k0))) / sc;
      err_sq = fma(q, q, err_sq);
    }
    return fmax(sqrt(err_sq / 4.0), 1.0e-10);
  }

  // Step-size factor from the error norm (integrate.j2:324-333).
  __device__ __forceinline__ static double growth(double err) {
    const double fac = 0.9 / cbrt(err);
    return fmax(0.2, fmin(fac, 6.0));
  }

  // ---- warp-cooperative attempt (tables + static warp schedules) ----
  static constexpr int NPART = 6;
  static constexpr int Q = NSLOTS;            // rates q_r, then q_i of the error norm
  static constexpr int D = NSLOTS + 4;     // partial derivatives
  static constexpr int COOP_SLOTS = NSLOTS + 4 + NPART;
  __device__ __forceinline__ static double acc_term(bool first, double acc, double coef, double t) {
    if (first) return coef == 1.0 ? t : (coef == -1.0 ? -t : coef * t);
    return coef == 1.0 ? acc + t : (coef == -1.0 ? acc - t : fma(coef, t, acc));
  }

  // F(y) into S[F..] for the state yv (S[Y..] or the stage state), cooperatively.
  template <class KA>
  __device__ __forceinline__ static void fun_coop(double* S, const double* yv, const KA& k, unsigned lane) {
    namespace T = coop;
    for (int r = lane; r < NR; r += 32) {
      double q = k(r);
      for (int e = T::r_off[r]; e < T::r_off[r + 1]; ++e) q = q * yv[T::r_y[e]];
      S[Q + r] = q;
    }
    __syncwarp();
    for (int i = lane; i < NV; i += 32) {
      double v = 0.0;
      for (int e = T::f_off[i]; e < T::f_off[i + 1]; ++e) v = acc_term(e == T::f_off[i], v, T::f_c[e], S[Q + T::f_r[e]]);
      S[F + i] = v;
    }
    __syncwarp();
  }

  // Run a static warp schedule (emitter/warp_schedule.py) on S: one
  // multiply-add, pivot multiply or reciprocal per lane and step, a warp
  // barrier between steps.  `out`, and `b` of a multiply-add, are offset by
  // base.  The next two steps' words are in flight while one executes.
  // Returns false if a reciprocal met a zero pivot.
  __device__ __forceinline__ static bool run_schedule(double* S, const unsigned long long* __restrict__ T,
                                                     int steps, int base, unsigned lane) {
    bool ok = true;
    unsigned long long cur = __ldg(T + lane);
    unsigned long long nxt = steps > 1 ? __ldg(T + 32 + lane) : 0ull;
    for (int s = 0; s < steps; ++s) {
      const unsigned long long nn = s + 2 < steps ? __ldg(T + (size_t)(s + 2) * 32 + lane) : 0ull;
      const int kind = (int)(cur >> 48) & 3;
      if (kind != 0) {
        const int out = (int)(cur & 0xffffu) + base;
        const int ia = (int)((cur >> 16) & 0xffffu);
        const int ib = (int)((cur >> 32) & 0xffffu) + (kind == 1 ? base : 0);
        const double vo = S[out];
        if (kind == 3) {
          ok = ok && (vo != 0.0);
          S[out] = 1.0 / vo;
        } else {
          // fma(-a, b, o) for a multiply-add; fma(o, b, -0.0) == o * b exactly.
          const double vb = S[ib];
          const double x = kind == 1 ? -S[ia] : vo;
          const double z = kind == 1 ? vo : -0.0;
          S[out] = fma(x, vb, z);
        }
      }
      __syncwarp();
      cur = nxt;
      nxt = nn;
    }
    return ok;
  }

  // Solve (LU) x = b in place on S[base..].
  __device__ __forceinline__ static void solve_coop(double* S, int base, unsigned lane) {
    run_schedule(S, coop::sv_fs, coop::SV_STEPS, base, lane);
  }

  // One attempt by a whole warp on the cell held in shared memory S
  // (NSLOTS + NR + NPART doubles).  Same values as attempt(); the error norm
  // is summed by lane 0 in species order.  Returns err on every lane.
  template <class KA>
  __device__ __forceinline__ static double attempt_coop(double* S, const KA& k, double h, int& status,
                                                       unsigned lane) {
    namespace T = coop;
    const double inv_g_dt = 1.0 / (GAMMA * h);
    // Jacobian partials, then W into the LU slots.
    for (int p = lane; p < NPART; p += 32) {
      double d = k(T::d_r[p]);
      for (int e = T::d_off[p]; e < T::d_off[p + 1]; ++e) {
        const int f = T::d_fac[e];
        d = d * (f < 0 ? T::d_lit[p] : S[Y + f]);
      }
      S[D + p] = d;
    }
    __syncwarp();
    for (int z = lane; z < T::N_LU_ZERO; z += 32) S[T::lu_zero[z]] = 0.0;
    for (int w = lane; w < T::NW; w += 32) {
      bool first = !T::w_diag[w];
      double v = T::w_diag[w] ? inv_g_dt : 0.0;
      for (int e = T::w_off[w]; e < T::w_off[w + 1]; ++e) {
        v = acc_term(first, v, T::w_c[e], S[D + T::w_p[e]]);
        first = false;
      }
      S[T::w_slot[w]] = v;
    }
    __syncwarp();
    // LU by the static warp schedule (fill-in slots were zeroed with W).
    const bool ok = run_schedule(S, T::lu_fs, T::LU_STEPS, 0, lane);
    if (__any_sync(0xffffffffu, !ok)) status |= 1;
    fun_coop(S, S + Y, k, lane);
    for (int i = lane; i < NV; i += 32) S[12 + i] = S[F + i];
    __syncwarp();
    solve_coop(S, 12, lane);
    // Stage state into the DY slots (free until the error block).
    for (int i = lane; i < NV; i += 32) S[DY + i] = S[Y + i] + S[12 + i];
    __syncwarp();
    fun_coop(S, S + DY, k, lane);
    const double c21 = -1.0156171083877703 / h;
    for (int i = lane; i < NV; i += 32) S[15 + i] = fma(c21, S[12 + i], S[F + i]);
    __syncwarp();
    solve_coop(S, 15, lane);
    const double c31 = 4.0759956452537702 / h;
    const double c32 = 9.20767942983308 / h;
    for (int i = lane; i < NV; i += 32) S[18 + i] = fma(c32, S[15 + i], fma(c31, S[12 + i], S[F + i]));
    __syncwarp();
    solve_coop(S, 18, lane);
    // Increment, and q_i^2 of the error norm into the rate slots.
    for (int i = lane; i < NV; i += 32) {
      const double k0 = S[12 + i];
      const double k1 = S[15 + i];
      const double k2 = S[18 + i];
      const double yi = S[Y + i];
      const double ynew = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, yi + k0));
      S[DY + i] = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, k0));
      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));
      S[Q + i] = (fma(0.22354069897811571, k2, fma(-2.9079558716805471, k1, 0.5 * k0))) / sc;
    }
    __syncwarp();
    double err = 0.0;
    if (lane == 0) {
      double err_sq = 0.0;
      for (int i = 0; i < NV; ++i) err_sq = fma(S[Q + i], S[Q + i], err_sq);
      err = fmax(sqrt(err_sq / 4.0), 1.0e-10);
    }
    return __shfl_sync(0xffffffffu, err, 0);
  }

  // ---- discrete adjoint of one accepted step ----
  static constexpr int LAM = 31;      // dL/dy
  static constexpr int KBAR = 34;    // stage adjoints, NSTAGE x NV
  static constexpr int FBAR = 43;    // adjoint of the pending stage tendency
  static constexpr int KB = 46;        // dL/dk accumulated
  static constexpr int NSLOTS_ADJ = 50;
  // Solve W^T x = b in place on [base, base + NV) with the stored LU of W.
  template <class SA>
  __device__ __forceinline__ static void solve_t(SA& S, const int base) {
    const double z0 = (S[base + 0]) * S[0];
    const double z1 = (fma(-S[1], z0, S[base + 1])) * S[4];
    const double z2 = (fma(-S[5], z1, fma(-S[2], z0, S[base + 2]))) * S[8];
    const double x2 = z2;
    S[base + 2] = x2;
    const double x1 = fma(-S[7], x2, z1);
    S[base + 1] = x1;
    const double x0 = fma(-S[6], x2, fma(-S[3], x1, z0));
    S[base + 0] = x0;
  }

  // u^T J(y) v terms of stage i: y in S[Y..], u in S[ub..], v = K_i in S[vb..].
  template <class SA, class KA>
  __device__ __forceinline__ static void adj_wterm(SA& S, const KA& k, const int ub, const int vb) {
    auto u = [&](int i) { return S[ub + i]; };
    const double y0 = S[Y + 0];
    const double v0 = S[vb + 0];
    const double y1 = S[Y + 1];
    const double v1 = S[vb + 1];
    const double y2 = S[Y + 2];
    const double v2 = S[vb + 2];
    { const double s = fma(2.0, u(1), -u(2));
      S[KB + 0] = fma(s, v2, S[KB + 0]);
      const double ks = k(0) * s;
    }
    { const double s = -u(1) - u(2) + u(0);
      S[KB + 1] = fma(s, (y2) * v1 + (y1) * v2, S[KB + 1]);
      const double ks = k(1) * s;
      S[LAM + 1] = fma(ks, v2, S[LAM + 1]);
      S[LAM + 2] = fma(ks, v1, S[LAM + 2]);
    }
    { const double s = -u(0) + u(1) + u(2);
      S[KB + 2] = fma(s, v0, S[KB + 2]);
      const double ks = k(2) * s;
    }
    { const double s = fma(2.0, u(2), -u(1) - u(0));
      S[KB + 3] = fma(s, (y1) * v0 + (y0) * v1, S[KB + 3]);
      const double ks = k(3) * s;
      S[LAM + 0] = fma(ks, v1, S[LAM + 0]);
      S[LAM + 1] = fma(ks, v0, S[LAM + 1]);
    }
  }

  // Adjoint of F_i = f(Y_i): Ybar = J(Y_i)^T Fbar, kbar += m_r(Y_i) (net_r.Fbar).
  // yv(i) supplies Y_i, ybar(j, x) receives Ybar_j.
  template <class SA, class KA, class YA, class OUT>
  __device__ __forceinline__ static void adj_fterm(SA& S, const KA& k, const YA& yv, OUT&& ybar) {
    auto fb = [&](int i) { return S[FBAR + i]; };
    const double y0 = yv(0);
    const double y1 = yv(1);
    const double y2 = yv(2);
    const double s0 = fma(2.0, fb(1), -fb(2));
    S[KB + 0] = fma(s0, y2, S[KB + 0]);
    const double s1 = -fb(1) - fb(2) + fb(0);
    S[KB + 1] = fma(s1, y1 * y2, S[KB + 1]);
    const double s2 = -fb(0) + fb(1) + fb(2);
    S[KB + 2] = fma(s2, y0, S[KB + 2]);
    const double s3 = fma(2.0, fb(2), -fb(1) - fb(0));
    S[KB + 3] = fma(s3, y0 * y1, S[KB + 3]);
    ybar(0, k(2) * s2 + k(3) * s3 * y1);
    ybar(1, k(1) * s1 * y2 + k(3) * s3 * y0);
    ybar(2, k(0) * s0 + k(1) * s1 * y1);
  }

  // Reverse of one accepted step of size h.  Requires the values attempt()
  // left in S for this step (LU, K_i) and y_n in S[Y..].
  template <class SA, class KA>
  __device__ __forceinline__ static void adjoint_step(SA& S, const KA& k, double h) {
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 0 + j] = 1.0 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 3 + j] = 6.1697947043828245 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 6 + j] = -0.42772256543218573 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 3
    solve_t(S, KBAR + 6);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 6, 18);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 6 + j];
    { const double cc = 4.0759956452537702 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 6 + q], S[KBAR + 0 + q]); }
    { const double cc = 9.20767942983308 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 3 + q] = fma(cc, S[KBAR + 6 + q], S[KBAR + 3 + q]); }
    // stage 2
    solve_t(S, KBAR + 3);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 3, 15);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 3 + j];
    { const double cc = -1.0156171083877703 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 3 + q], S[KBAR + 0 + q]); }
    adj_fterm(S, k, [&](int q) { return S[Y + q] + S[12 + q]; },
              [&](int j, double x) { S[LAM + j] += x; S[KBAR + 0 + j] = fma(1.0, x, S[KBAR + 0 + j]); });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 1
    solve_t(S, KBAR + 0);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 0, 12);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 0 + j];
    adj_fterm(S, k, [&](int q) { return S[Y + q]; },
              [&](int j, double x) { S[LAM + j] += x; });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
  }
};

}  // namespace mkpp_chapman

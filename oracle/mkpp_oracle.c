/*
 * CPU oracle (TEST INFRASTRUCTURE ONLY): a plain-C restatement of the MKPP
 * per-cell Rosenbrock solve.  It is the checker for the GPU kernels in
 * tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py; no
 * product code path links, loads or calls it.
 *
 * It runs the reference's *full* N x N system (fixed species included) from
 * the tables of a plan JSON, following the generated code step by step:
 *   - W assembly            src/mkpp/templates/solver_variants/integrate.j2:103-107
 *   - factorize_plan        src/mkpp/templates/device_impl/supernodal_factorize.hpp.j2:10-31
 *                           (value = w; value -= l*r ...; lu = value / diag)
 *   - solve_plan            src/mkpp/templates/device_impl/supernodal_solve.hpp.j2:10-42
 *   - stages Y/rhs/K        integrate.j2:144-263 (A, C, NewF of the tableau,
 *                           coefficients src/mkpp/rosenbrock.py:27-134)
 *   - error norm            integrate.j2:265-322 (divides by N incl. fixed species)
 *   - step controller       integrate.j2:71-84, 324-379
 * The species tendencies and Jacobian are mass-action sums over reactions
 * with the rate constants evaluated once per integrate() call (the
 * reference recomputes them inside each expression,
 * src/mkpp/templates/device_impl/rates.hpp.j2 and jacobian.hpp.j2); the
 * rate-constant values and their fixed-species derivatives are inputs.
 *
 * Build: gcc -O2 -fopenmp -shared -fPIC mkpp_oracle.c -o libmkpp_oracle.so -lm
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_MAX_STAGES 6

typedef struct {
  int ns, nr;
  const int* fixed;        /* [ns] */
  const int* perm;         /* [ns] logical -> physical */
  /* reactions */
  const int* react_off;    /* [nr+1] variable reactants (physical index, power) */
  const int* react_sp;
  const int* react_pow;
  const int* net_off;      /* [nr+1] net stoichiometry on variable species */
  const int* net_sp;
  const double* net_c;
  const int* dk_off;       /* [nr+1] d k_r / d C_fixed entries */
  const int* dk_sp;
  /* Jacobian slots: physical (i, j) -> slot, dense ns*ns map, -1 if absent */
  int nj;
  const int* jslot_of;
  /* W (compact, logical order) */
  int nw;
  const int* w_diag;       /* [nw] 1 if on the diagonal */
  const int* w_jslot;      /* [nw] J slot or -1 */
  /* LU schedule */
  int nlu, nops;
  const int* op_out, *op_w, *op_begin, *op_end, *op_diag;
  const int* prod_l, *prod_r;
  const int* lower_off, *lower_col, *lower_slot;
  const int* upper_off, *upper_col, *upper_slot;
  const int* diag;
  /* tableau */
  int stages;
  double gamma, elo;
  double A[ORACLE_MAX_STAGES * ORACLE_MAX_STAGES];
  double C[ORACLE_MAX_STAGES * ORACLE_MAX_STAGES];
  double M[ORACLE_MAX_STAGES], E[ORACLE_MAX_STAGES];
  int newf[ORACLE_MAX_STAGES];
  const double* atol, *rtol;  /* physical order */
} oracle_plan;

typedef struct {
  double* J;     /* [nj] */
  double* W;     /* [nw] */
  double* LU;    /* [nlu] */
  double* F;     /* [ns] physical */
  double* Fl;    /* [ns] logical */
  double* S;     /* [ns] logical state */
  double* Y;     /* [ns] physical stage state */
  double* K;     /* [stages * ns] logical */
  double* rhs;   /* [ns] */
  double* work;  /* [ns] */
} oracle_scratch;

/* Mass-action tendencies, physical order (fixed species stay 0). */
static void fun(const oracle_plan* p, const double* y, const double* k, double* F) {
  for (int s = 0; s < p->ns; ++s) F[s] = 0.0;
  for (int r = 0; r < p->nr; ++r) {
    double q = k[r];
    for (int e = p->react_off[r]; e < p->react_off[r + 1]; ++e)
      for (int w = 0; w < p->react_pow[e]; ++w) q *= y[p->react_sp[e]];
    for (int e = p->net_off[r]; e < p->net_off[r + 1]; ++e) F[p->net_sp[e]] += p->net_c[e] * q;
  }
}

/* Jacobian at the compact physical slots, fixed-species columns included. */
static void jac(const oracle_plan* p, const double* y, const double* k, const double* dk, double* J) {
  for (int s = 0; s < p->nj; ++s) J[s] = 0.0;
  for (int r = 0; r < p->nr; ++r) {
    for (int a = p->react_off[r]; a < p->react_off[r + 1]; ++a) {
      /* d/dC_a of k * prod y^nu */
      double d = k[r] * (double)p->react_pow[a];
      for (int w = 0; w < p->react_pow[a] - 1; ++w) d *= y[p->react_sp[a]];
      for (int b = p->react_off[r]; b < p->react_off[r + 1]; ++b) {
        if (b == a) continue;
        for (int w = 0; w < p->react_pow[b]; ++w) d *= y[p->react_sp[b]];
      }
      const int col = p->react_sp[a];
      for (int e = p->net_off[r]; e < p->net_off[r + 1]; ++e)
        J[p->jslot_of[p->net_sp[e] * p->ns + col]] += p->net_c[e] * d;
    }
    for (int f = p->dk_off[r]; f < p->dk_off[r + 1]; ++f) {
      double d = dk[f];
      for (int b = p->react_off[r]; b < p->react_off[r + 1]; ++b)
        for (int w = 0; w < p->react_pow[b]; ++w) d *= y[p->react_sp[b]];
      const int col = p->dk_sp[f];
      for (int e = p->net_off[r]; e < p->net_off[r + 1]; ++e)
        J[p->jslot_of[p->net_sp[e] * p->ns + col]] += p->net_c[e] * d;
    }
  }
}

/* factorize_plan (supernodal_factorize.hpp.j2:10-31). */
static void factorize(const oracle_plan* p, const double* w, double* lu) {
  for (int o = 0; o < p->nops; ++o) {
    double value = p->op_w[o] >= 0 ? w[p->op_w[o]] : 0.0;
    for (int q = p->op_begin[o]; q < p->op_end[o]; ++q) value -= lu[p->prod_l[q]] * lu[p->prod_r[q]];
    lu[p->op_out[o]] = p->op_diag[o] >= 0 ? value / lu[p->op_diag[o]] : value;
  }
}

/* solve_plan (supernodal_solve.hpp.j2:10-42). */
static void solve(const oracle_plan* p, const double* lu, const double* rhs, double* work, double* sol) {
  const int n = p->ns;
  for (int row = 0; row < n; ++row) {
    work[row] = rhs[row];
    for (int e = p->lower_off[row]; e < p->lower_off[row + 1]; ++e) work[row] -= lu[p->lower_slot[e]] * work[p->lower_col[e]];
  }
  for (int row = n - 1; row >= 0; --row) {
    sol[row] = work[row];
    for (int e = p->upper_off[row]; e < p->upper_off[row + 1]; ++e) sol[row] -= lu[p->upper_slot[e]] * sol[p->upper_col[e]];
    sol[row] /= lu[p->diag[row]];
  }
}

/* One attempt from the physical state `state`; returns the error norm and
 * leaves the stage vectors K in scratch. */
static double attempt(const oracle_plan* p, oracle_scratch* s, const double* state, const double* k,
                      const double* dk, double dt) {
  const int n = p->ns;
  const double inv_g_dt = 1.0 / (p->gamma * dt);
  for (int i = 0; i < n; ++i) s->S[i] = state[p->perm[i]];
  jac(p, state, k, dk, s->J);
  for (int w = 0; w < p->nw; ++w) {
    const double base = p->w_diag[w] ? inv_g_dt : 0.0;
    s->W[w] = p->w_jslot[w] >= 0 ? base - s->J[p->w_jslot[w]] : base;
  }
  factorize(p, s->W, s->LU);
  int have_f = 0;
  for (int st = 0; st < p->stages; ++st) {
    if (p->newf[st]) {
      if (st == 0) {
        fun(p, state, k, s->F);
      } else {
        /* Y_st = S + sum_j A_{st,j} K_j, written back in physical order */
        for (int i = 0; i < n; ++i) {
          double v = s->S[i];
          for (int j = 0; j < st; ++j) {
            const double a = p->A[st * ORACLE_MAX_STAGES + j];
            if (a == 0.0) continue;
            v = (a == 1.0) ? v + s->K[j * n + i] : v + a * s->K[j * n + i];
          }
          s->Y[p->perm[i]] = v;
        }
        fun(p, s->Y, k, s->F);
      }
      for (int i = 0; i < n; ++i) s->Fl[i] = s->F[p->perm[i]];
      have_f = 1;
    }
    (void)have_f;
    for (int i = 0; i < n; ++i) {
      double v = s->Fl[i];
      for (int j = 0; j < st; ++j) {
        const double c = p->C[st * ORACLE_MAX_STAGES + j];
        if (c == 0.0) continue;
        v = v + (c / dt) * s->K[j * n + i];
      }
      s->rhs[i] = v;
    }
    solve(p, s->LU, s->rhs, s->work, s->K + st * n);
  }
  double err_sq = 0.0;
  for (int i = 0; i < n; ++i) {
    double ynew = s->S[i];
    double yerr = 0.0;
    int first = 1;
    for (int j = 0; j < p->stages; ++j) {
      const double m = p->M[j];
      if (m != 0.0) ynew = (m == 1.0) ? ynew + s->K[j * n + i] : ynew + m * s->K[j * n + i];
    }
    for (int j = 0; j < p->stages; ++j) {
      const double e = p->E[j];
      if (e == 0.0) continue;
      const double term = (e == 1.0) ? s->K[j * n + i] : e * s->K[j * n + i];
      yerr = first ? term : yerr + term;
      first = 0;
    }
    const int phys = p->perm[i];
    const double ymax = fmax(fabs(state[phys]), fabs(ynew));
    const double sci = p->atol[phys] + p->rtol[phys] * ymax;
    err_sq += (yerr / sci) * (yerr / sci);
  }
  double err = sqrt(err_sq / n);
  return fmax(err, 1.0e-10);
}

/* state += sum_j M_j K_j (integrate.j2 accept block). */
static void accept_step(const oracle_plan* p, oracle_scratch* s, double* state) {
  const int n = p->ns;
  for (int i = 0; i < n; ++i) {
    double inc = 0.0;
    int first = 1;
    for (int j = 0; j < p->stages; ++j) {
      const double m = p->M[j];
      if (m == 0.0) continue;
      const double term = (m == 1.0) ? s->K[j * n + i] : m * s->K[j * n + i];
      inc = first ? term : inc + term;
      first = 0;
    }
    state[p->perm[i]] += inc;
  }
}

static double growth(const oracle_plan* p, double err) {
  double factor;
  if (p->elo == 2.0) factor = 0.9 / sqrt(err);
  else if (p->elo == 3.0) factor = 0.9 / cbrt(err);
  else factor = 0.9 * pow(err, -1.0 / p->elo);
  return fmax(0.2, fmin(factor, 6.0));
}

static int alloc_scratch(const oracle_plan* p, oracle_scratch* s) {
  const int n = p->ns;
  s->J = malloc(sizeof(double) * (p->nj > 0 ? p->nj : 1));
  s->W = malloc(sizeof(double) * p->nw);
  s->LU = malloc(sizeof(double) * p->nlu);
  s->F = malloc(sizeof(double) * n);
  s->Fl = malloc(sizeof(double) * n);
  s->S = malloc(sizeof(double) * n);
  s->Y = malloc(sizeof(double) * n);
  s->K = malloc(sizeof(double) * n * p->stages);
  s->rhs = malloc(sizeof(double) * n);
  s->work = malloc(sizeof(double) * n);
  return s->J && s->W && s->LU && s->F && s->Fl && s->S && s->Y && s->K && s->rhs && s->work;
}

static void free_scratch(oracle_scratch* s) {
  free(s->J); free(s->W); free(s->LU); free(s->F); free(s->Fl);
  free(s->S); free(s->Y); free(s->K); free(s->rhs); free(s->work);
}

/*
 * Integrate ncells cells `steps` times over dt seconds each.
 *   conc   [ns][ncells] in/out (LayoutLeft, cell innermost)
 *   ktab   [nr][ncells] rate constants
 *   dktab  [ndk][ncells] fixed-species derivatives of the rate constants
 * Optional: status/accepted/rejected [ncells]; log_* record (h, accepted) of
 * every attempt at [a * ncells + c] up to log_cap.  With replay_n != NULL the
 * step sequence is not chosen by the controller but read from replay_h /
 * replay_acc (same layout), replay_n[c] attempts for cell c.
 * dt_carry (optional, [ncells] in/out): step-size carry-over across
 * integrate() calls, a non-parity option of this build (the reference
 * restarts every call at dt_total * seed and lists carried step estimates as
 * future work, SCALING_OPTIMIZATION_REPORT.md:27-29).  A call starts at
 * fmin(carry, dt_total) where carry > 0 and finite, else at dt_total * seed.
 * What carries into the next call (and, after the last one, is written
 * back) is the controller's proposal after the call's last accepted step,
 * or, if that step was cut short to end at dt_total, the step size the
 * controller wanted before the cut.
 * Returns the number of cells with a non-zero status.
 */
int mkpp_oracle_integrate(const oracle_plan* p, int ncells, double* conc, const double* ktab,
                          const double* dktab, int ndk, double dt_total, int steps, double seed,
                          int max_attempts, int nthreads, int* status, int* accepted, int* rejected,
                          double* log_h, unsigned char* log_acc, int* log_n, int log_cap,
                          const double* replay_h, const unsigned char* replay_acc, const int* replay_n,
                          double* dt_carry) {
  int failures = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel reduction(+ : failures)
  {
    oracle_scratch s;
    double* state = malloc(sizeof(double) * p->ns);
    double* k = malloc(sizeof(double) * (p->nr > 0 ? p->nr : 1));
    double* dk = malloc(sizeof(double) * (ndk > 0 ? ndk : 1));
    const int ok_alloc = alloc_scratch(p, &s) && state && k && dk;
#pragma omp for schedule(dynamic, 16)
    for (int c = 0; c < ncells; ++c) {
      int st = 0, nacc = 0, nrej = 0, logged = 0;
      if (!ok_alloc) { st = 4; goto done; }
      for (int i = 0; i < p->ns; ++i) state[i] = conc[(size_t)i * ncells + c];
      for (int r = 0; r < p->nr; ++r) k[r] = ktab[(size_t)r * ncells + c];
      for (int e = 0; e < ndk; ++e) dk[e] = dktab[(size_t)e * ncells + c];
      for (int i = 0; i < p->ns; ++i) if (!isfinite(state[i])) st = 2;
      for (int r = 0; r < p->nr; ++r) if (!isfinite(k[r])) st = 2;
      if (st) goto done;
      if (replay_n) {
        for (int a = 0; a < replay_n[c]; ++a) {
          const double h = replay_h[(size_t)a * ncells + c];
          (void)attempt(p, &s, state, k, dk, h);
          if (replay_acc[(size_t)a * ncells + c]) { accept_step(p, &s, state); ++nacc; } else { ++nrej; }
        }
      } else {
        double carry = dt_carry ? dt_carry[c] : 0.0;
        for (int step = 0; step < steps && !st; ++step) {
          /* integrate.j2:71-84 */
          const double h_min = dt_total * 1.0e-15;
          double t = 0.0;
          double dtc = (carry > 0.0 && isfinite(carry)) ? fmin(carry, dt_total) : dt_total * seed;
          int reject_last = 0, reject_more = 0, attempts = 0;
          double dtc_last = 0.0, want_last = 0.0;
          double want = dtc; /* the controller's step before the end-of-call cut */
          while (t < dt_total) {
            if (attempts >= max_attempts) { st = 3; break; }
            want = dtc;
            dtc = fmin(dtc, dt_total - t);
            const double err = attempt(p, &s, state, k, dk, dtc);
            const double factor = growth(p, err);
            ++attempts;
            const int acc = err <= 1.0;
            if (log_h && logged < log_cap) {
              log_h[(size_t)logged * ncells + c] = dtc;
              log_acc[(size_t)logged * ncells + c] = (unsigned char)acc;
              ++logged;
            }
            if (acc) {
              accept_step(p, &s, state);
              dtc_last = dtc;
              want_last = want;
              t += dtc;
              double next_dt = fmax(h_min, fmin(dtc * factor, dt_total));
              if (reject_last) next_dt = fmin(next_dt, dtc);
              reject_last = 0;
              reject_more = 0;
              dtc = next_dt;
              ++nacc;
            } else {
              dtc *= reject_more ? 0.1 : factor;
              reject_more = reject_last;
              reject_last = 1;
              ++nrej;
            }
          }
          /* a last step cut to reach dt_total says nothing about the step
             size: carry the controller's step before the cut instead */
          if (dt_carry) carry = (dtc_last < want_last) ? want_last : dtc;
        }
        if (dt_carry) dt_carry[c] = carry;
      }
      for (int i = 0; i < p->ns; ++i) conc[(size_t)i * ncells + c] = state[i];
      if (!st) for (int i = 0; i < p->ns; ++i) if (!isfinite(state[i])) st = 4;
    done:
      if (status) status[c] = st;
      if (accepted) accepted[c] = nacc;
      if (rejected) rejected[c] = nrej;
      if (log_n) log_n[c] = logged;
      failures += st != 0;
    }
    free_scratch(&s);
    free(state);
    free(k);
    free(dk);
  }
  return failures;
}

/* Species tendencies F and the compact Jacobian values of one state per cell. */
int mkpp_oracle_eval(const oracle_plan* p, int ncells, const double* conc, const double* ktab,
                     const double* dktab, int ndk, double* F_out, double* J_out) {
  double* y = malloc(sizeof(double) * p->ns);
  double* k = malloc(sizeof(double) * (p->nr > 0 ? p->nr : 1));
  double* dk = malloc(sizeof(double) * (ndk > 0 ? ndk : 1));
  double* F = malloc(sizeof(double) * p->ns);
  double* J = malloc(sizeof(double) * (p->nj > 0 ? p->nj : 1));
  if (!y || !k || !dk || !F || !J) return -1;
  for (int c = 0; c < ncells; ++c) {
    for (int i = 0; i < p->ns; ++i) y[i] = conc[(size_t)i * ncells + c];
    for (int r = 0; r < p->nr; ++r) k[r] = ktab[(size_t)r * ncells + c];
    for (int e = 0; e < ndk; ++e) dk[e] = dktab[(size_t)e * ncells + c];
    fun(p, y, k, F);
    jac(p, y, k, dk, J);
    if (F_out) for (int i = 0; i < p->ns; ++i) F_out[(size_t)i * ncells + c] = F[i];
    if (J_out) for (int s = 0; s < p->nj; ++s) J_out[(size_t)s * ncells + c] = J[s];
  }
  free(y); free(k); free(dk); free(F); free(J);
  return 0;
}

// Mechanism-independent Rosenbrock driver kernels (sm_103a, FP64).
//
// Data layout in HBM (all LayoutLeft, cell index innermost, so a warp's 32
// lanes touch 32 consecutive doubles of the same species / reaction row):
//   conc   [NS][ncells]   species concentrations, updated in place
//   param  [NP][ncells]   runtime parameters (photolysis J, external rates)
//   ktab   [NR][ncells]   rate constants, written by rate_constant_kernel
//   temp/rho/rh/clw [ncells]
//
// One thread owns one cell.  The per-cell controller reproduces
// SolverKernels::integrate (src/mkpp/templates/solver_variants/integrate.j2:71-84,
// 324-379): dt0 = dt_total * seed, h_min = dt_total * 1e-15,
// dt = min(dt, dt_total - t), factor clamp [0.2, 6], no growth right after a
// rejection, tenfold cut after two consecutive rejections.  Unlike the
// reference, every integrate() call is bounded by max_attempts; a cell that
// hits the bound stops with CELL_ERR_CONVERGENCE_FAILURE instead of spinning.
#pragma once
#include <type_traits>

#include "mkpp_device.cuh"

namespace mkpp {

struct LaunchArgs {
  int ncells;
  int steps;                 // integrate() calls per cell with the same forcing
  double dt;                 // dt_total of each call [s]
  double seed;               // initial_step_seed
  int max_attempts;          // per integrate() call
  double* conc;              // [NS][ncells]
  const double* ktab;        // [NR][ncells] (host step 0)
  size_t k_step_stride;      // doubles between the rate tables of consecutive host
                             // steps (0: the same rate constants for every step)
  int* status;               // [ncells] or null
  int* n_accept;             // [ncells] or null (accumulated over steps)
  int* n_reject;             // [ncells] or null
  unsigned int* queue;       // persistent kernel work counter (zeroed before launch)
  const int* order;          // persistent kernel: queue position -> cell, or null (identity)
  // Hand-off of slow cells to the warp-cooperative kernel: a cell whose
  // attempts (over all its host steps so far) reach defer_after (> 0) is
  // parked in defer[] (controller state) with its state written back to conc.
  struct Deferred* defer;
  unsigned int* defer_count;
  int defer_after;
  // Optional per-attempt log for step-sequence replay in the CPU oracle:
  // entry a of cell c at [a * ncells + c]; log_n[c] = attempts recorded.
  double* log_h;
  unsigned char* log_acc;
  int* log_n;
  int log_cap;
  // Tail parking (integrate_persistent_kernel<Mech, MINB, true>): once the
  // queue is drained and at most tail_cells cells are still on lanes, a cell
  // with at least tail_after attempts is parked as well.  active counts the
  // cells on lanes (zeroed before launch).
  unsigned int* active;
  int tail_after;
  unsigned int tail_cells;
  // Step-size carry-over across integrate() calls (null: off, the
  // reference's controller): dt_carry[c] > 0 starts the cell's first call
  // at that step size instead of dt * seed, each later call of the launch
  // starts from the previous call's carry, and the last call's carry is
  // written back (Controller::carry_out).
  double* dt_carry;
  // Split launch (integrate_split_kernel): the first split_cells entries of
  // order are integrated by whole warps on the SMs with id < split_sms, the
  // persistent body takes its cells from order[split_cells..]; split_next is
  // the warps' work counter (zeroed before launch).
  int split_cells;
  int split_sms;
  unsigned int* split_next;
};

// Controller state of a parked cell (see LaunchArgs::defer).
struct Deferred {
  int cell, step, attempts, nacc, nrej, flags;  // flags: 1 reject_last, 2 reject_more, 4 zero pivot, 8 cut
  double t, dt, want;
};

struct RateArgs {
  int ncells;
  const double* conc;        // [NS][ncells]  (fixed species are read here)
  const double* param;       // [NP][ncells] or null (zeros)
  const double* temp;        // [ncells] or null (compile-time environment)
  const double* rho;         // [ncells] or null
  const double* rh;          // [ncells] or null (0.5)
  const double* clw;         // [ncells] or null (0.0)
  double* ktab;              // [NR][ncells]
  int* status;               // [ncells] or null: non-finite inputs are flagged
};

// ---------------------------------------------------------------------------
// Rate constants: one thread per cell, k_r for every reaction.
// ---------------------------------------------------------------------------
struct ZeroRow {
  __device__ __forceinline__ double operator()(int) const { return 0.0; }
};

template <class Mech>
__global__ void __launch_bounds__(128, 1) rate_constant_kernel(RateArgs a) {
  const size_t n = (size_t)a.ncells;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const double T = a.temp ? a.temp[c] : Mech::ENV_T;
    const double RHO = a.rho ? a.rho[c] : Mech::ENV_RHO;
    const double RH = a.rh ? a.rh[c] : 0.5;
    const double CLW = a.clw ? a.clw[c] : 0.0;
    CellRow fix{a.conc + c, n};
    CellRowOut k{a.ktab + c, n};
    if (a.param) {
      CellRow P{a.param + c, n};
      Mech::rate_constants(P, fix, T, RHO, RH, CLW, k);
    } else {
      ZeroRow P;
      Mech::rate_constants(P, fix, T, RHO, RH, CLW, k);
    }
    if (a.status) {
      bool ok = finite(T) && finite(RHO);
#pragma unroll 1
      for (int s = 0; s < Mech::NS; ++s) ok = ok && finite(a.conc[c + n * s]);
#pragma unroll 1
      for (int r = 0; r < Mech::NR; ++r) ok = ok && finite(a.ktab[c + n * r]);
      a.status[c] = ok ? CELL_SUCCESS : CELL_ERR_NON_FINITE_STATE;
    }
  }
}

// ---------------------------------------------------------------------------
// Per-cell working storage (LU factors, state, stage vectors).
//
// Small mechanisms keep it in a private array that the compiler promotes to
// registers.  Large ones use a slice of a global-memory tile owned by the
// thread's block, laid out [slot][thread] so that a warp's access to one slot
// is 32 consecutive doubles and every slot address is an immediate offset
// from the thread's base pointer.
// ---------------------------------------------------------------------------
constexpr int kBlock = 128;
constexpr int kRegisterSlots = 96;

template <int N>
struct RegStore {
  double v[N];
  __device__ __forceinline__ double& operator[](int s) { return v[s]; }
};

struct TileStore {
  double* __restrict__ p;
  __device__ __forceinline__ double& operator[](int s) const { return p[(size_t)s * kBlock]; }
};

template <class Mech>
struct StoreFor {
  static constexpr bool kTile = Mech::NSLOTS > kRegisterSlots;
  using type = typename std::conditional<kTile, TileStore, RegStore<(kTile ? 1 : Mech::NSLOTS)>>::type;
  // Global scratch bytes per block (zero when the store lives in registers).
  static constexpr size_t block_bytes = kTile ? (size_t)Mech::NSLOTS * kBlock * sizeof(double) : 0;
};

template <class Mech>
__device__ __forceinline__ TileStore make_store(double* scratch, TileStore*, unsigned block = blockIdx.x) {
  return TileStore{scratch + (size_t)block * Mech::NSLOTS * kBlock + threadIdx.x};
}
template <class Mech, int N>
__device__ __forceinline__ RegStore<N> make_store(double*, RegStore<N>*, unsigned = 0) {
  return RegStore<N>{};
}

// ---------------------------------------------------------------------------
// Per-cell controller state and one controller step.
// ---------------------------------------------------------------------------
struct Controller {
  double t, dt, dt_total, h_min;
  double want;       // the step size chosen before the end-of-call cut
  bool reject_last, reject_more;
  bool cut;          // the last attempt was cut short to end at dt_total
  int attempts;

  // carry > 0 and finite: start at fmin(carry, total) (step-size carry-over,
  // off by default); otherwise at total * seed as integrate.j2:80 does.
  __device__ __forceinline__ void start(double total, double seed, double carry = 0.0) {
    dt_total = total;
    h_min = total * 1.0e-15;
    t = 0.0;
    dt = (carry > 0.0 && finite(carry)) ? fmin(carry, total) : total * seed;
    want = dt;
    reject_last = reject_more = cut = false;
    attempts = 0;
  }
  __device__ __forceinline__ bool running() const { return t < dt_total; }
  // Step size of the next attempt (integrate.j2:85: dt = min(dt, dt_total - t)).
  __device__ __forceinline__ double next_h() {
    want = dt;
    cut = dt_total - t < dt;
    dt = fmin(dt, dt_total - t);
    return dt;
  }
  // Step size carried into the next call once this one has ended: the
  // proposal after its last accepted step, or, when that step was cut short
  // to end at dt_total, the step size wanted before the cut.
  __device__ __forceinline__ double carry_out() const { return cut ? want : dt; }
  // Accept/reject bookkeeping (integrate.j2:335-379); returns true on accept.
  template <class Mech>
  __device__ __forceinline__ bool update(double err) {
    const double factor = Mech::growth(err);
    ++attempts;
    if (err <= 1.0) {
      t += dt;
      double next_dt = fmax(h_min, fmin(dt * factor, dt_total));
      if (reject_last) next_dt = fmin(next_dt, dt);
      reject_last = false;
      reject_more = false;
      dt = next_dt;
      return true;
    }
    dt *= reject_more ? 0.1 : factor;
    reject_more = reject_last;
    reject_last = true;
    return false;
  }
};

// A cell skipped because its input is not finite made no attempt in this
// call: its counts say so, rather than keeping an earlier call's.
__device__ __forceinline__ void clear_counts(const LaunchArgs& a, size_t c) {
  if (a.n_accept) a.n_accept[c] = 0;
  if (a.n_reject) a.n_reject[c] = 0;
}

template <class Mech, class SA>
__device__ __forceinline__ void load_state(const double* conc, size_t c, size_t n, SA& S) {
#pragma unroll
  for (int i = 0; i < Mech::NV; ++i) S[Mech::Y + i] = conc[c + n * Mech::var_phys(i)];
}

template <class Mech, class SA>
__device__ __forceinline__ void store_state(double* conc, size_t c, size_t n, SA& S) {
#pragma unroll
  for (int i = 0; i < Mech::NV; ++i) conc[c + n * Mech::var_phys(i)] = S[Mech::Y + i];
}

template <class Mech, class SA>
__device__ __forceinline__ bool state_finite(SA& S) {
  bool ok = true;
#pragma unroll
  for (int i = 0; i < Mech::NV; ++i) ok = ok && finite(S[Mech::Y + i]);
  return ok;
}

// Rate constants of host step `step` of cell c into the working storage, so
// that every attempt reads them from the cell's own slots.
template <class Mech, class SA>
__device__ __forceinline__ void load_rates(const LaunchArgs& a, size_t c, int step, SA& S) {
  const double* __restrict__ k = a.ktab + (size_t)step * a.k_step_stride + c;
  const size_t n = (size_t)a.ncells;
#pragma unroll 8
  for (int r = 0; r < Mech::NR; ++r) S[Mech::KT + r] = __ldg(k + (size_t)r * n);
}

template <class Mech, class SA>
__device__ __forceinline__ void apply_increment(SA& S) {
#pragma unroll
  for (int i = 0; i < Mech::NV; ++i) S[Mech::Y + i] += S[Mech::DY + i];
}

// Final status of a cell: non-finite state, attempt cap, zero pivot seen.
// A zero pivot does not stop the cell: like the reference (which has no
// singularity check) it runs on, and a non-finite result is reported as
// CELL_ERR_NUMERICAL_FAILURE; a finite result after a zero pivot keeps
// CELL_ERR_SINGULAR_MATRIX.
template <class Mech, class SA>
__device__ __forceinline__ int final_status(SA& S, bool capped, bool zero_pivot) {
  if (!state_finite<Mech>(S)) return CELL_ERR_NUMERICAL_FAILURE;
  if (capped) return CELL_ERR_CONVERGENCE_FAILURE;
  return zero_pivot ? CELL_ERR_SINGULAR_MATRIX : CELL_SUCCESS;
}

// One cell, `steps` integrate() calls; the plain kernel's per-cell body.
template <class Mech, class SA>
__device__ __forceinline__ int integrate_cell(SA& S, const LaunchArgs& a, size_t c, int& nacc, int& nrej) {
  const size_t n = (size_t)a.ncells;
  int logged = 0;
  bool capped = false, zero_pivot = false;
  nacc = nrej = 0;
  double carry = a.dt_carry ? a.dt_carry[c] : 0.0;
  for (int step = 0; step < a.steps && !capped; ++step) {
    load_rates<Mech>(a, c, step, S);
    auto k = [&](int r) { return S[Mech::KT + r]; };
    Controller ctl;
    ctl.start(a.dt, a.seed, carry);
    while (ctl.running()) {
      if (ctl.attempts >= a.max_attempts) {
        capped = true;
        break;
      }
      const double h = ctl.next_h();
      int st = 0;
      const double err = Mech::attempt(S, k, h, st);
      zero_pivot |= st != 0;
      const bool acc = ctl.update<Mech>(err);
      if (a.log_h && logged < a.log_cap) {
        a.log_h[(size_t)logged * n + c] = h;
        a.log_acc[(size_t)logged * n + c] = acc ? 1 : 0;
        ++logged;
      }
      if (acc) {
        apply_increment<Mech>(S);
        ++nacc;
      } else {
        ++nrej;
      }
    }
    if (a.dt_carry) carry = ctl.carry_out();
  }
  if (a.dt_carry) a.dt_carry[c] = carry;
  if (a.log_n) a.log_n[c] = logged;
  return final_status<Mech>(S, capped, zero_pivot);
}

// MINB is the launch-bounds minimum of resident blocks per SM: 2 lets each
// thread use up to 255 registers (2 blocks of 128 fit), 4 caps it at 128 so
// that 4 blocks can be resident, trading spills for latency hiding.
// ---------------------------------------------------------------------------
// Plain form: a fixed grid, thread t integrates cells t, t + T, t + 2T, ...
// (T = grid threads) one after the other.  A warp runs until its slowest
// lane is done, so lanes with easy cells idle while stiff ones finish.
// ---------------------------------------------------------------------------
template <class Mech, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) integrate_plain_kernel(LaunchArgs a, double* scratch) {
  using Store = typename StoreFor<Mech>::type;
  Store S = make_store<Mech>(scratch, (Store*)nullptr);
  const size_t n = (size_t)a.ncells;
  const size_t T = (size_t)gridDim.x * kBlock;
  for (size_t c = blockIdx.x * (size_t)kBlock + threadIdx.x; c < n; c += T) {
    if (a.status && a.status[c] != CELL_SUCCESS) {
      clear_counts(a, c);
      continue;
    }
    load_state<Mech>(a.conc, c, n, S);
    int nacc, nrej;
    const int status = integrate_cell<Mech>(S, a, c, nacc, nrej);
    store_state<Mech>(a.conc, c, n, S);
    if (a.status) a.status[c] = status;
    if (a.n_accept) a.n_accept[c] = nacc;
    if (a.n_reject) a.n_reject[c] = nrej;
  }
}

// ---------------------------------------------------------------------------
// Persistent form: a grid sized to the SMs; every lane pulls cells from a
// device work counter and refills itself as soon as its cell has finished,
// so a warp's lanes stay busy even when cells need very different numbers
// of attempts.  All lanes run the same attempt code on different cells.
// ---------------------------------------------------------------------------
// The persistent kernel's body for one block (its tile is scratch tile
// `block`); integrate_split_kernel runs it on the SMs it does not reserve.
template <class Mech, bool TAIL>
__device__ __forceinline__ void persistent_body(const LaunchArgs& a, double* scratch, unsigned block) {
  using Store = typename StoreFor<Mech>::type;
  Store S = make_store<Mech>(scratch, (Store*)nullptr, block);
  const size_t n = (size_t)a.ncells;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  long long cell = -1;       // -1: needs work; >= n: queue exhausted
  int step = 0, nacc = 0, nrej = 0;
  bool flagged = false;      // cell rejected by the input checks: leave it untouched
  bool capped = false, zero_pivot = false;
  bool left = false;         // (TAIL) the lane's cell finished or was parked last iteration
  Controller ctl;
  ctl.start(a.dt, a.seed);
  for (;;) {
    if constexpr (TAIL) {
      const unsigned gone = __ballot_sync(0xffffffffu, left);
      if (gone && (int)lane == __ffs(gone) - 1) atomicSub(a.active, (unsigned)__popc(gone));
      left = false;
    }
    const bool need = cell < 0;
    const unsigned want = __ballot_sync(0xffffffffu, need);
    if (want) {
      const int leader = __ffs(want) - 1;
      unsigned base = 0;
      if ((int)lane == leader) base = atomicAdd(a.queue, (unsigned)__popc(want));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        cell = (long long)base + __popc(want & lt_mask) + a.split_cells;
        if (cell < (long long)n && a.order) cell = a.order[cell];
        if (cell < (long long)n) {
          flagged = a.status && a.status[cell] != CELL_SUCCESS;
          step = 0;
          nacc = nrej = 0;
          capped = zero_pivot = false;
          if (!flagged) {
            load_state<Mech>(a.conc, (size_t)cell, n, S);
            load_rates<Mech>(a, (size_t)cell, 0, S);
          }
          ctl.start(a.dt, a.seed, a.dt_carry && !flagged ? a.dt_carry[cell] : 0.0);
        }
      }
      if constexpr (TAIL) {
        const unsigned got = __ballot_sync(0xffffffffu, need && cell < (long long)n);
        if (got && (int)lane == __ffs(got) - 1) atomicAdd(a.active, (unsigned)__popc(got));
      }
    }
    const bool active = cell >= 0 && cell < (long long)n;
    if (__ballot_sync(0xffffffffu, active) == 0u) break;
    if (!active) continue;
    bool done = flagged;
    if (!done) {
      if (ctl.attempts >= a.max_attempts) {
        capped = true;
        done = true;
      } else {
        auto k = [&](int r) { return S[Mech::KT + r]; };
        const double h = ctl.next_h();
        int st = 0;
        const double err = Mech::attempt(S, k, h, st);
        zero_pivot |= st != 0;
        if (ctl.update<Mech>(err)) {
          apply_increment<Mech>(S);
          ++nacc;
        } else {
          ++nrej;
        }
        if (!ctl.running()) {
          if (++step < a.steps) {
            ctl.start(a.dt, a.seed, a.dt_carry ? ctl.carry_out() : 0.0);
            load_rates<Mech>(a, (size_t)cell, step, S);
          } else {
            done = true;
          }
        } else if ((a.defer_after > 0 && nacc + nrej >= a.defer_after) ||
                   (TAIL && a.tail_after > 0 && nacc + nrej >= a.tail_after && ((nacc + nrej) & 15) == 0 &&
                    __ldcg(a.queue) >= (unsigned)(n - a.split_cells) && __ldcg(a.active) <= a.tail_cells)) {
          // Too slow for one lane, or one of the last cells on lanes: park
          // the cell for the cooperative kernel.
          const unsigned slot = atomicAdd(a.defer_count, 1u);
          Deferred d;
          d.cell = (int)cell;
          d.step = step;
          d.attempts = ctl.attempts;
          d.nacc = nacc;
          d.nrej = nrej;
          d.flags = (ctl.reject_last ? 1 : 0) | (ctl.reject_more ? 2 : 0) | (zero_pivot ? 4 : 0) | (ctl.cut ? 8 : 0);
          d.t = ctl.t;
          d.dt = ctl.dt;
          d.want = ctl.want;
          a.defer[slot] = d;
          store_state<Mech>(a.conc, (size_t)cell, n, S);
          cell = -1;
          left = true;
          continue;
        }
      }
    }
    if (done) {
      const size_t cc = (size_t)cell;
      if (!flagged) {
        store_state<Mech>(a.conc, cc, n, S);
        if (a.dt_carry) a.dt_carry[cc] = ctl.carry_out();
        if (a.status) a.status[cc] = final_status<Mech>(S, capped, zero_pivot);
      }
      // (a flagged cell's counts are zero: it made no attempt)
      if (a.n_accept) a.n_accept[cc] = nacc;
      if (a.n_reject) a.n_reject[cc] = nrej;
      cell = -1;
      left = true;
    }
  }
}

template <class Mech, int MINB, bool TAIL = false>
__global__ void __launch_bounds__(kBlock, MINB) integrate_persistent_kernel(LaunchArgs a, double* scratch) {
  persistent_body<Mech, TAIL>(a, scratch, blockIdx.x);
}


// ---------------------------------------------------------------------------
// Cooperative form for parked cells: a whole warp integrates one cell at a
// time, the cell's working set in shared memory, each attempt spread over
// the lanes by the level schedules of Mech::attempt_coop.  It resumes the
// parked controller state exactly, and attempt_coop reproduces attempt's
// arithmetic, so a parked cell ends bit-identical to an unparked one.
// ---------------------------------------------------------------------------
constexpr int kCoopWarps = 4;

// One cell on a whole warp, from the controller state ctl at host step
// `step` (attempt and accept counts so far in nacc, nrej) to the end of its
// last host step; the cell's state is in S[Y..] already.  Writes the state,
// status, counts and carried step size back.
template <class Mech>
__device__ __forceinline__ void coop_integrate_cell(const LaunchArgs& a, double* S, unsigned lane, size_t c,
                                                    Controller& ctl, int step, int nacc, int nrej,
                                                    bool zero_pivot) {
  const size_t n = (size_t)a.ncells;
  bool capped = false;
  for (; step < a.steps;) {
    for (int r = lane; r < Mech::NR; r += 32) S[Mech::KT + r] = a.ktab[(size_t)step * a.k_step_stride + c + n * r];
    __syncwarp();
    auto k = [&](int r) { return S[Mech::KT + r]; };
    while (ctl.running()) {
      if (ctl.attempts >= a.max_attempts) {
        capped = true;
        break;
      }
      const double h = ctl.next_h();
      int st = 0;
      const double err = Mech::attempt_coop(S, k, h, st, lane);
      zero_pivot |= st != 0;
      if (ctl.update<Mech>(err)) {
        for (int i = lane; i < Mech::NV; i += 32) S[Mech::Y + i] += S[Mech::DY + i];
        __syncwarp();
        ++nacc;
      } else {
        ++nrej;
      }
    }
    if (capped || ++step >= a.steps) break;
    ctl.start(a.dt, a.seed, a.dt_carry ? ctl.carry_out() : 0.0);
  }
  bool fin = true;
  for (int i = lane; i < Mech::NV; i += 32) fin = fin && finite(S[Mech::Y + i]);
  fin = __all_sync(0xffffffffu, fin);
  for (int i = lane; i < Mech::NV; i += 32) a.conc[c + n * Mech::var_phys(i)] = S[Mech::Y + i];
  if (lane == 0) {
    if (a.dt_carry) a.dt_carry[c] = ctl.carry_out();
    const int status = !fin ? CELL_ERR_NUMERICAL_FAILURE
                            : (capped ? CELL_ERR_CONVERGENCE_FAILURE
                                      : (zero_pivot ? CELL_ERR_SINGULAR_MATRIX : CELL_SUCCESS));
    if (a.status) a.status[c] = status;
    if (a.n_accept) a.n_accept[c] = nacc;
    if (a.n_reject) a.n_reject[c] = nrej;
  }
  __syncwarp();
}

template <class Mech>
__global__ void __launch_bounds__(kCoopWarps * 32, 1) integrate_coop_kernel(LaunchArgs a) {
  extern __shared__ double smem[];
  const unsigned lane = threadIdx.x & 31u;
  const unsigned wib = threadIdx.x >> 5;
  const unsigned wpb = blockDim.x >> 5;  // warps launched per block (<= kCoopWarps)
  double* S = smem + (size_t)wib * Mech::COOP_SLOTS;
  const size_t n = (size_t)a.ncells;
  const unsigned count = *a.defer_count;
  for (unsigned idx = blockIdx.x * wpb + wib; idx < count; idx += gridDim.x * wpb) {
    const Deferred d = a.defer[idx];
    const size_t c = (size_t)d.cell;
    for (int i = lane; i < Mech::NV; i += 32) S[Mech::Y + i] = a.conc[c + n * Mech::var_phys(i)];
    __syncwarp();
    Controller ctl;
    ctl.start(a.dt, a.seed);
    ctl.t = d.t;
    ctl.dt = d.dt;
    ctl.want = d.want;
    ctl.attempts = d.attempts;
    ctl.reject_last = d.flags & 1;
    ctl.reject_more = (d.flags & 2) != 0;
    ctl.cut = (d.flags & 8) != 0;
    coop_integrate_cell<Mech>(a, S, lane, c, ctl, d.step, d.nacc, d.nrej, (d.flags & 4) != 0);
  }
}

// ---------------------------------------------------------------------------
// Split form: one launch in which the blocks on the first split_sms SMs
// (by the SM id the hardware reports) integrate the first split_cells cells
// of the order, the most expensive ones, each on a whole warp from its
// start, while the blocks on the other SMs run the persistent body over the
// rest of the order.  A warp finishes a SAPRC99 attempt ~3x sooner than a
// lane when its SM runs no lanes, so the cells that would set the end of
// the launch on lanes finish earlier; reserving whole SMs keeps the
// persistent blocks' FP64 work off those warps' SMs.  Each warp takes the
// next cell from a.split_next.  Results are bit-identical to the other
// forms (attempt_coop reproduces attempt).  A warp's store is a slice of its
// block's scratch tile (unused by the persistent body there), so the launch
// needs no shared memory and the persistent blocks keep the whole L1.
// ---------------------------------------------------------------------------
template <class Mech>
__global__ void __launch_bounds__(kBlock, 2) integrate_split_kernel(LaunchArgs a, double* scratch) {
  static_assert(kCoopWarps * 32 == kBlock, "a split block is kCoopWarps warps");
  static_assert((size_t)kCoopWarps * Mech::COOP_SLOTS <= StoreFor<Mech>::block_bytes / sizeof(double),
                "the warps' stores fit in the block's scratch tile");
  unsigned smid;
  asm("mov.u32 %0, %%smid;" : "=r"(smid));  // the SM this block runs on
  if (smid >= (unsigned)a.split_sms) {
    persistent_body<Mech, false>(a, scratch, blockIdx.x);
    return;
  }
  const unsigned lane = threadIdx.x & 31u;
  double* S = scratch + (size_t)blockIdx.x * Mech::NSLOTS * kBlock + (size_t)(threadIdx.x >> 5) * Mech::COOP_SLOTS;
  const size_t n = (size_t)a.ncells;
  // Every pass takes a new counter value, so a warp makes at most
  // split_cells + 1 passes.
  for (int pass = 0; pass <= a.split_cells; ++pass) {
    unsigned idx = 0;
    if (lane == 0) idx = atomicAdd(a.split_next, 1u);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= (unsigned)a.split_cells) break;
    const long long cell = a.order[idx];
    if (cell < 0 || cell >= (long long)n) continue;  // an order entry out of range names no cell
    const size_t c = (size_t)cell;
    if (a.status && a.status[c] != CELL_SUCCESS) {
      if (lane == 0) clear_counts(a, c);
      continue;
    }
    for (int i = lane; i < Mech::NV; i += 32) S[Mech::Y + i] = a.conc[c + n * Mech::var_phys(i)];
    __syncwarp();
    Controller ctl;
    ctl.start(a.dt, a.seed, a.dt_carry ? a.dt_carry[c] : 0.0);
    coop_integrate_cell<Mech>(a, S, lane, c, ctl, 0, 0, 0, false);
  }
}

// ---------------------------------------------------------------------------
// Differentiation: forward with checkpoints at accepted steps, the discrete
// adjoint sweep over them, and a replay of a frozen step sequence.
// Checkpoint layout (cell index innermost): the state before accepted step s
// at y[(s * NV + i) * ncells + c], its step size at h[s * ncells + c], the
// number of accepted steps at n[c].
// ---------------------------------------------------------------------------
struct CheckpointArgs {
  int cap;            // accepted steps a cell may record
  double* y;
  double* h;
  int* n;
  // Recorded steps of cell c as the sweeps read them: the forward writes at
  // most cap, and a count handed in through the device entries is clamped
  // to [0, cap] so that no sweep reads past the checkpoint arrays.
  __device__ __forceinline__ int count(size_t c) const { return min(max(n[c], 0), cap); }
};

template <int N>
struct StoreN {
  static constexpr bool kTile = N > kRegisterSlots;
  using type = typename std::conditional<kTile, TileStore, RegStore<(kTile ? 1 : N)>>::type;
  static constexpr size_t block_bytes = kTile ? (size_t)N * kBlock * sizeof(double) : 0;
  __device__ __forceinline__ static type make(double* scratch) {
    type s{};
    if constexpr (kTile) s.p = scratch + (size_t)blockIdx.x * N * kBlock + threadIdx.x;
    return s;
  }
};

// One integrate() call per cell (plain form) that records (y_n, h) at every
// accepted step.  Same arithmetic as integrate_plain_kernel.
template <class Mech>
__global__ void __launch_bounds__(kBlock, 2) integrate_checkpoint_kernel(LaunchArgs a, CheckpointArgs ck,
                                                                         double* scratch) {
  using SN = StoreN<Mech::NSLOTS>;
  typename SN::type S = SN::make(scratch);
  const size_t n = (size_t)a.ncells;
  const size_t T = (size_t)gridDim.x * kBlock;
  for (size_t c = blockIdx.x * (size_t)kBlock + threadIdx.x; c < n; c += T) {
    if (a.status && a.status[c] != CELL_SUCCESS) {
      ck.n[c] = 0;  // no accepted step to revisit
      clear_counts(a, c);
      continue;
    }
    load_state<Mech>(a.conc, c, n, S);
    load_rates<Mech>(a, c, 0, S);
    auto k = [&](int r) { return S[Mech::KT + r]; };
    Controller ctl;
    ctl.start(a.dt, a.seed);
    int nacc = 0, nrej = 0, cnt = 0;
    bool capped = false, zero_pivot = false, overflow = false;
    while (ctl.running()) {
      if (ctl.attempts >= a.max_attempts) {
        capped = true;
        break;
      }
      const double h = ctl.next_h();
      int st = 0;
      const double err = Mech::attempt(S, k, h, st);
      zero_pivot |= st != 0;
      if (ctl.update<Mech>(err)) {
        if (cnt >= ck.cap) {
          overflow = true;
          break;
        }
#pragma unroll 4
        for (int i = 0; i < Mech::NV; ++i) ck.y[((size_t)cnt * Mech::NV + i) * n + c] = S[Mech::Y + i];
        ck.h[(size_t)cnt * n + c] = h;
        ++cnt;
        apply_increment<Mech>(S);
        ++nacc;
      } else {
        ++nrej;
      }
    }
    store_state<Mech>(a.conc, c, n, S);
    ck.n[c] = cnt;
    const int status = overflow ? CELL_ERR_CHECKPOINT_OVERFLOW : final_status<Mech>(S, capped, zero_pivot);
    if (a.status) a.status[c] = status;
    if (a.n_accept) a.n_accept[c] = nacc;
    if (a.n_reject) a.n_reject[c] = nrej;
  }
}

// Applies the recorded accepted steps (frozen step sequence) to conc.
template <class Mech>
__global__ void __launch_bounds__(kBlock, 2) integrate_replay_kernel(LaunchArgs a, CheckpointArgs ck,
                                                                     double* scratch) {
  using SN = StoreN<Mech::NSLOTS>;
  typename SN::type S = SN::make(scratch);
  const size_t n = (size_t)a.ncells;
  const size_t T = (size_t)gridDim.x * kBlock;
  for (size_t c = blockIdx.x * (size_t)kBlock + threadIdx.x; c < n; c += T) {
    load_state<Mech>(a.conc, c, n, S);
    load_rates<Mech>(a, c, 0, S);
    auto k = [&](int r) { return S[Mech::KT + r]; };
    const int cnt = ck.count(c);
    for (int s = 0; s < cnt; ++s) {
      int st = 0;
      (void)Mech::attempt(S, k, ck.h[(size_t)s * n + c], st);
      apply_increment<Mech>(S);
    }
    store_state<Mech>(a.conc, c, n, S);
  }
}

struct AdjointArgs {
  int ncells;
  const double* ktab;      // [NR][ncells]
  const double* lam;       // [NS][ncells]  dL/dy at the end of the call
  double* grad_conc;       // [NS][ncells]  dL/dy at the start (fixed species 0)
  double* grad_k;          // [NR][ncells]  dL/dk
};

// Reverse sweep: for each accepted step, last to first, recompute the step
// from its checkpoint with attempt() (bit-identical to the forward) and apply
// Mech::adjoint_step.
template <class Mech>
__global__ void __launch_bounds__(kBlock, 2) adjoint_kernel(AdjointArgs a, CheckpointArgs ck, double* scratch) {
  using SN = StoreN<Mech::NSLOTS_ADJ>;
  typename SN::type S = SN::make(scratch);
  const size_t n = (size_t)a.ncells;
  const size_t T = (size_t)gridDim.x * kBlock;
  for (size_t c = blockIdx.x * (size_t)kBlock + threadIdx.x; c < n; c += T) {
#pragma unroll 4
    for (int r = 0; r < Mech::NR; ++r) {
      S[Mech::KT + r] = __ldg(a.ktab + (size_t)r * n + c);
      S[Mech::KB + r] = 0.0;
    }
#pragma unroll 4
    for (int i = 0; i < Mech::NV; ++i) S[Mech::LAM + i] = a.lam[c + n * Mech::var_phys(i)];
    auto k = [&](int r) { return S[Mech::KT + r]; };
    for (int s = ck.count(c) - 1; s >= 0; --s) {
#pragma unroll 4
      for (int i = 0; i < Mech::NV; ++i) S[Mech::Y + i] = ck.y[((size_t)s * Mech::NV + i) * n + c];
      const double h = ck.h[(size_t)s * n + c];
      int st = 0;
      (void)Mech::attempt(S, k, h, st);
      Mech::adjoint_step(S, k, h);
    }
    for (int i = 0; i < Mech::NS; ++i) a.grad_conc[c + n * i] = 0.0;
#pragma unroll 4
    for (int i = 0; i < Mech::NV; ++i) a.grad_conc[c + n * Mech::var_phys(i)] = S[Mech::LAM + i];
#pragma unroll 4
    for (int r = 0; r < Mech::NR; ++r) a.grad_k[c + n * r] = S[Mech::KB + r];
  }
}

struct TangentArgs {
  int ncells;
  const double* ktab;      // [NR][ncells]
  const double* dconc0;    // [NS][ncells]  tangent of conc at the start (fixed species ignored)
  const double* dk;        // [NR][ncells]  tangent of the rate constants, or null for none
  double* dconc;           // [NS][ncells]  tangent of conc at the end (fixed species 0)
};

// Tangent sweep: for each accepted step, first to last, recompute the step
// from its checkpoint with attempt() (bit-identical to the forward) and carry
// the tangent through Mech::tlm_step.  tlm_step addresses the store through
// its program's slot numbers, so the store is always the per-block tile.
template <class Mech>
__global__ void __launch_bounds__(kBlock, 2) tangent_kernel(TangentArgs a, CheckpointArgs ck, double* scratch) {
  TileStore S{scratch + (size_t)blockIdx.x * Mech::NSLOTS_TLM * kBlock + threadIdx.x};
  const size_t n = (size_t)a.ncells;
  const size_t T = (size_t)gridDim.x * kBlock;
  for (size_t c = blockIdx.x * (size_t)kBlock + threadIdx.x; c < n; c += T) {
#pragma unroll 4
    for (int r = 0; r < Mech::NR; ++r) {
      S[Mech::KT + r] = __ldg(a.ktab + (size_t)r * n + c);
      S[Mech::DKR + r] = a.dk ? __ldg(a.dk + (size_t)r * n + c) : 0.0;
    }
#pragma unroll 4
    for (int i = 0; i < Mech::NV; ++i) S[Mech::DYT + i] = a.dconc0[c + n * Mech::var_phys(i)];
    auto k = [&](int r) { return S[Mech::KT + r]; };
    const int cnt = ck.count(c);
    for (int s = 0; s < cnt; ++s) {
#pragma unroll 4
      for (int i = 0; i < Mech::NV; ++i) S[Mech::Y + i] = ck.y[((size_t)s * Mech::NV + i) * n + c];
      const double h = ck.h[(size_t)s * n + c];
      int st = 0;
      (void)Mech::attempt(S, k, h, st);
      Mech::tlm_step(S, k, h);
    }
    for (int i = 0; i < Mech::NS; ++i) a.dconc[c + n * i] = 0.0;
#pragma unroll 4
    for (int i = 0; i < Mech::NV; ++i) a.dconc[c + n * Mech::var_phys(i)] = S[Mech::DYT + i];
  }
}

}  // namespace mkpp

"""The emitted GPU arithmetic, run on the host (CPU).

The per-thread attempt of each generated header (mkpp_gb300/generated/<m>.cuh)
is compiled for the host through tests/hostsim/.  The CUDA qualifiers become
plain C++, and -ffp-contract=off lets only explicit fma() calls fuse, as in
the GPU build (--fmad=false).  For one attempt on seeded cells:
* the two emitted forms agree bit for bit: the per-thread attempt's stage
  vectors and factorised LU slots equal those of the cooperative kernel's
  stage programs, executed in program order with exactly rounded fma;
* the accepted step agrees with the oracle's step with the same step size
  forced, per species to 1e-9 (|oracle| + atol), the GPU parity gate.  The
  two formulations differ at round-off, and a single step amplifies that by
  cond(W): measured, the difference tracks eps * cond(W) (Chapman 5e-16,
  small_strato 1e-12 at cond 1e5, SAPRC99 2.5e-10 at cond 3e8).  So the
  step size per mechanism keeps cond(W) below ~1e9 on these cells.
SAPRC99 runs with its three 1e33-1e37 1/s rate constants moderated to 1e3,
as in the GPU forced-step test, and so do saprc99_mini and saprcnov (the
same Troe rates), which get the first two checks too.
"""

import ctypes as C
from fractions import Fraction

from pathlib import Path

import hostsim_lib
import numpy as np
import pytest

from mkpp_gb300 import workloads
from mkpp_gb300.emitter import cuda_emitter
from mkpp_gb300.emitter import warp_schedule as ws
from mkpp_gb300.emitter.plan import load
from oracle.oracle import Oracle

MECHS = ["chapman", "small_strato", "saprc99"]
# Further mechanisms the reference ships, checked for the forward step.
EXTRA = ["saprc99_mini", "saprcnov", "chapman_rodas3", "small_strato_rodas3"]
# Step sizes of the oracle comparison: cond(W) at most ~10, 1.5e5, 3e8 and
# (TS1) 2.3e7.  TS1 at 1 s has cond(W) 1.8e10, and with atol 1 molec/cm3 in
# mol/m3 its trace species then differ by up to 7e-9 of their value.
H_ORACLE = {"chapman": 1e-4, "small_strato": 1e-4, "saprc99": 1e-6, "ts1": 1e-2, "saprc99_mini": 1e-6,
            "saprcnov": 1e-6, "chapman_rodas3": 1e-4, "small_strato_rodas3": 1e-4}
# Rate constants of the shipped mechanisms that reach 1e29-1e41 1/s (Troe k0
# evaluated as A exp(+C/T)); moderated to 1e3 as in the GPU forced-step test.
EXTREME = {"saprc99": (11, 32, 69), "ts1": (375, 376, 383, 394, 397, 402), "saprc99_mini": (7,),
           "saprcnov": (10, 31, 57)}


class _Libs(dict):
    """Hostsim libraries by mechanism, each compiled on first use."""

    def __init__(self, out):
        super().__init__()
        self.out = out

    def __missing__(self, mech):
        self[mech] = hostsim_lib.compile(self.out, mech)
        return self[mech]


@pytest.fixture(scope="module")
def hostsim(tmp_path_factory):
    return _Libs(tmp_path_factory.mktemp("hostsim"))


_layout = hostsim_lib.layout


def _xfma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _run_programs(progs, S):
    S = list(S)
    for ops in progs:
        for kind, out, a, b, c, neg in ops:
            if kind == ws.RCP:
                S[out] = 1.0 / S[out]
            else:
                S[out] = _xfma(-S[a] if neg else S[a], S[b], S[c])
    return np.array(S)


def _case(mech, n=4):
    w = workloads.make(mech, n)
    o = Oracle(mech)
    k, dk = o.rate_constants(w.conc, w.temp, w.rho, w.rh, None, w.param)
    for r in EXTREME.get(mech, ()):
        k[r] = np.minimum(k[r], 1e3)
    return w, o, k, dk


@pytest.mark.parametrize("mech", MECHS + EXTRA)
def test_per_thread_attempt_equals_cooperative_programs(hostsim, mech):
    lib = hostsim[mech]
    L = _layout(lib)
    plan = load(mech)
    cuda_emitter.emit_mechanism(plan)
    progs, _, info = plan._coop_programs
    assert (info["Y"], info["K0"], info["FS"], info["DY"], info["KT"]) == (L["Y"], L["K0"], L["F"], L["DY"], L["KT"])
    w, o, k, _ = _case(mech)
    nv, nlu = L["NV"], len(plan.lu_slots)
    h = 10.0
    for c in range(w.ncells):
        y = np.ascontiguousarray(w.conc[plan.var_phys, c])
        kc = np.ascontiguousarray(k[:, c])
        S = np.zeros(L["NSLOTS"])
        S[L["Y"]:L["Y"] + nv] = y
        st = C.c_int(0)
        lib.hostsim_attempt(S.ctypes.data, kc.ctypes.data, h, C.byref(st))
        P = np.zeros(info["slots"])
        P[info["Y"]:info["Y"] + nv] = y
        P[info["KT"]:info["KT"] + len(kc)] = kc
        CB = info["CB"]
        P[CB:CB + 4] = (-0.0, 0.0, 1.0, 1.0 / (plan.tableau["Gamma"][0] * h))
        for (s_, j), slot in info["cterm_slot"].items():
            P[slot] = info["C"][(s_ - 1) * (s_ - 2) // 2 + j - 1] / h
        for v, slot in info["literals"].items():
            P[slot] = v
        P = _run_programs(progs, P)
        K = slice(L["K0"], L["K0"] + L["NSTAGE"] * nv)
        assert st.value == 0
        assert np.array_equal(S[K], P[K])
        assert np.array_equal(S[:nlu], P[:nlu])


@pytest.mark.parametrize("mech", MECHS + EXTRA)
def test_per_thread_step_matches_oracle_with_forced_step(hostsim, mech):
    _forced_step_vs_oracle(hostsim[mech], mech)


def test_ts1_table_step_matches_oracle_with_forced_step(hostsim):
    _forced_step_vs_oracle(hostsim["ts1"], "ts1")


def _forced_step_vs_oracle(lib, mech):
    L = _layout(lib)
    plan = load(mech)
    w, o, k, dk = _case(mech, 8)
    nv = L["NV"]
    h = H_ORACLE[mech]
    for c in range(w.ncells):
        y = np.ascontiguousarray(w.conc[plan.var_phys, c])
        kc = np.ascontiguousarray(k[:, c])
        S = np.zeros(L["NSLOTS"])
        S[L["Y"]:L["Y"] + nv] = y
        st = C.c_int(0)
        lib.hostsim_attempt(S.ctypes.data, kc.ctypes.data, h, C.byref(st))
        assert st.value == 0
        ynew = y + S[L["DY"]:L["DY"] + nv]
        rep = o.integrate(w.conc[:, c:c + 1].copy(), h, k=k[:, c:c + 1].copy(), dk=dk[:, c:c + 1].copy(),
                          temp=w.temp[c:c + 1], rho=w.rho[c:c + 1], rh=w.rh[c:c + 1], param=w.param[:, c:c + 1],
                          replay=(np.array([[h]]), np.array([[1]], np.uint8), np.array([1], np.int32)))
        ref = rep["conc"][plan.var_phys, 0]
        atol = np.array(o.raw["atol"])[plan.var_phys]
        assert np.all(np.abs(ynew - ref) <= 1e-9 * (np.abs(ref) + atol))


_compile = hostsim_lib.compile


@pytest.mark.parametrize("mech", MECHS)
def test_table_attempt_equals_unrolled_attempt(hostsim, mech, tmp_path):
    """The table-driven per-thread attempt (emitted for mechanisms too large
    to unroll, here forced) ends bit-identical to the unrolled one: state
    increment, stage vectors, factorised LU and error norm."""
    plan = load(mech)
    (tmp_path / f"{mech}.cuh").write_text(cuda_emitter.emit_mechanism(plan, table=True))
    table = _compile(tmp_path, mech, include_first=tmp_path)
    unrolled = hostsim[mech]
    Lt, Lu = _layout(table), _layout(unrolled)
    assert Lt["NSLOTS"] > Lu["NSLOTS"] and all(Lt[k] == Lu[k] for k in ("Y", "K0", "F", "DY", "KT", "NV"))
    w, o, k, _ = _case(mech)
    nv = Lu["NV"]
    for h in (1e-4, 10.0):
        for c in range(w.ncells):
            y = w.conc[plan.var_phys, c]
            kc = np.ascontiguousarray(k[:, c])
            out = []
            for lib, L in ((unrolled, Lu), (table, Lt)):
                S = np.zeros(L["NSLOTS"])
                S[L["Y"]:L["Y"] + nv] = y
                st = C.c_int(0)
                err = lib.hostsim_attempt(S.ctypes.data, kc.ctypes.data, h, C.byref(st))
                out.append((S[:L["KT"]].copy(), err, st.value))
            assert np.array_equal(out[0][0], out[1][0])
            assert out[0][1] == out[1][1] and out[0][2] == out[1][2]


def test_ts1_table_attempt_equals_its_programs(hostsim):
    """TS1 (210 species, 49299 LU multiply-adds) is emitted table-driven: its
    host-compiled per-thread attempt gives the stage vectors and LU of its
    stage programs executed in program order with exactly rounded fma."""
    mech = "ts1"
    lib = hostsim[mech]
    L = _layout(lib)
    plan = load(mech)
    cuda_emitter.emit_mechanism(plan)
    progs, _, info = plan._coop_programs
    w, o, k, _ = _case(mech, 1)
    nv, nlu = L["NV"], len(plan.lu_slots)
    h = 1e-4
    y = np.ascontiguousarray(w.conc[plan.var_phys, 0])
    kc = np.ascontiguousarray(k[:, 0])
    S = np.zeros(L["NSLOTS"])
    S[L["Y"]:L["Y"] + nv] = y
    st = C.c_int(0)
    lib.hostsim_attempt(S.ctypes.data, kc.ctypes.data, h, C.byref(st))
    P = np.zeros(info["slots"])
    P[info["Y"]:info["Y"] + nv] = y
    P[info["KT"]:info["KT"] + len(kc)] = kc
    CB = info["CB"]
    P[CB:CB + 4] = (-0.0, 0.0, 1.0, 1.0 / (plan.tableau["Gamma"][0] * h))
    for (s_, j), slot in info["cterm_slot"].items():
        P[slot] = info["C"][(s_ - 1) * (s_ - 2) // 2 + j - 1] / h
    for v, slot in info["literals"].items():
        P[slot] = v
    P = _run_programs(progs, P)
    K = slice(L["K0"], L["K0"] + L["NSTAGE"] * nv)
    assert np.isfinite(S[K]).all()
    assert np.array_equal(S[K], P[K])
    assert np.array_equal(S[:nlu], P[:nlu])


def _adj_layout(lib):
    v = (C.c_int * 3)()
    lib.hostsim_adj_layout(v)
    return dict(zip(("LAM", "KB", "NSLOTS_ADJ"), list(v)))


def _host_adjoint(lib, y, k, h, lam):
    """(dL/dy_n, dL/dk, status) of one step through the emitted adjoint."""
    L, A = _layout(lib), _adj_layout(lib)
    nv, nr = L["NV"], L["NR"]
    S = np.zeros(A["NSLOTS_ADJ"])
    S[L["Y"]:L["Y"] + nv] = y
    S[A["LAM"]:A["LAM"] + nv] = lam
    st = C.c_int(0)
    kc = np.ascontiguousarray(k)
    lib.hostsim_adjoint.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    lib.hostsim_adjoint(S.ctypes.data, kc.ctypes.data, h, C.byref(st))
    return S[A["LAM"]:A["LAM"] + nv].copy(), S[A["KB"]:A["KB"] + nr].copy(), st.value


@pytest.mark.parametrize("mech", MECHS)
def test_table_adjoint_equals_unrolled_adjoint(hostsim, mech, tmp_path):
    """The table-driven adjoint step (the reverse-step program, here forced
    on a mechanism that is normally unrolled) gives dL/dy_n and dL/dk
    bit-identical to the unrolled adjoint step."""
    plan = load(mech)
    (tmp_path / f"{mech}.cuh").write_text(cuda_emitter.emit_mechanism(plan, table=True))
    table = _compile(tmp_path, mech, include_first=tmp_path)
    w, o, k, _ = _case(mech)
    rng = np.random.default_rng(5)
    for h in (1e-4, 10.0):
        for c in range(w.ncells):
            y = w.conc[plan.var_phys, c]
            lam = rng.uniform(-1.0, 1.0, plan.n_var)
            a = _host_adjoint(hostsim[mech], y, k[:, c], h, lam)
            b = _host_adjoint(table, y, k[:, c], h, lam)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2] == 0


def test_ts1_table_adjoint_matches_dense_adjoint(hostsim):
    """TS1's table-driven adjoint of one step against the dense FP64 CPU
    adjoint (oracle/adjoint_ref.py), scale-free: |dg * x| <= 1e-8 max|g * x|
    for x = y_n and x = k (measured: 1e-17 and 1e-11)."""
    from oracle.adjoint_ref import DenseModel

    lib = hostsim["ts1"]
    plan = load("ts1")
    dm = DenseModel("ts1")
    w, o, k, _ = _case("ts1", 2)
    rng = np.random.default_rng(5)
    for h in (1e-2, 1.0):
        for c in range(w.ncells):
            y = w.conc[plan.var_phys, c]
            kc = k[:, c]
            lam = rng.uniform(-1.0, 1.0, plan.n_var) / np.maximum(np.abs(y), 1.0)
            g, gk, st = _host_adjoint(lib, y, kc, h, lam)
            assert st == 0
            _, tape = dm.forward(y, kc, [h])
            g0, gk0 = dm.adjoint(kc, tape, lam)
            assert np.abs((g - g0) * y).max() <= 1e-8 * np.abs(g0 * y).max()
            assert np.abs((gk - gk0) * kc).max() <= 1e-8 * np.abs(gk0 * kc).max()


_host_tlm = hostsim_lib.tangent_step


def _jacobians(lib, mech, y, k, h):
    """d y_new / d y and d y_new / d k of one step: columns from the tangent
    (dy or dk a unit vector) and rows from the adjoint (lambda a unit
    vector)."""
    nv, nr = len(y), len(k)
    tl_y, tl_k = np.zeros((nv, nv)), np.zeros((nv, nr))
    for j in range(nv):
        e = np.zeros(nv)
        e[j] = 1.0
        tl_y[:, j] = _host_tlm(lib, y, k, h, e, np.zeros(nr))[0]
    for r in range(nr):
        e = np.zeros(nr)
        e[r] = 1.0
        tl_k[:, r] = _host_tlm(lib, y, k, h, np.zeros(nv), e)[0]
    ad_y, ad_k = np.zeros((nv, nv)), np.zeros((nv, nr))
    for i in range(nv):
        e = np.zeros(nv)
        e[i] = 1.0
        ad_y[i, :], ad_k[i, :], _ = _host_adjoint(lib, y, k, h, e)
    return tl_y, tl_k, ad_y, ad_k


def _column_error(a, b):
    """max over columns of |a - b| / max|b| in that column."""
    scale = np.maximum(np.abs(b).max(axis=0), 1e-300)
    return (np.abs(a - b).max(axis=0) / scale).max()


ROS3 = [m for m in MECHS + EXTRA + ["ts1"] if not m.endswith("_rodas3")]
RODAS3 = [m for m in EXTRA if m.endswith("_rodas3")]


@pytest.mark.parametrize("mech", ROS3)
def test_tangent_is_the_transpose_of_the_adjoint(hostsim, mech):
    """For one step, the emitted tangent (tlm_step) and adjoint
    (adjoint_step) give the same derivative: every column of d y_new/d y and
    d y_new/d k from the tangent equals the adjoint's to 64 eps cond(W) of
    the column's largest entry, W = I/(gamma h) - J the stage matrix.  Both
    are exact derivatives of the same rounded map taken in opposite
    accumulation orders, so they differ by round-off amplified by cond(W);
    measured 0.01-4.4 eps cond(W) over the four mechanisms at h = 1e-3 and 1
    (SAPRC99 at h = 1: 1.8e-8 with cond(W) = 3.3e9).  (The reference's own
    tests check the same transpose identity, test_adjoint_identity.py.)"""
    from oracle.adjoint_ref import DenseModel

    lib = hostsim[mech]
    plan = load(mech)
    dm = DenseModel(mech)
    w, o, k, _ = _case(mech, 1)
    y = w.conc[plan.var_phys, 0]
    kc = k[:, 0]
    for h in (1e-3, 1.0):
        W = np.eye(plan.n_var) / (dm.g * h) - dm.J(y, kc)
        bound = 64 * np.finfo(float).eps * max(np.linalg.cond(W), 1.0)
        tl_y, tl_k, ad_y, ad_k = _jacobians(lib, mech, y, kc, h)
        assert _column_error(tl_y, ad_y) <= bound
        assert _column_error(tl_k, ad_k) <= bound


def _step_mp(dm, y, k, h, digits=60):
    """One step of the dense model's tableau in `digits`-digit arithmetic
    (mpmath): the exact map the FP64 kernels round."""
    import mpmath as mp

    mp.mp.dps = digits
    nv, nr = dm.nv, dm.nr
    S = mp.matrix(dm.S.tolist())

    def mono(yv):
        out = [mp.mpf(1)] * nr
        for r, e in enumerate(dm.expo):
            for j, pw in e.items():
                out[r] *= yv[j] ** pw
        return out

    def dmono(yv):
        D = mp.zeros(nr, nv)
        for r, e in enumerate(dm.expo):
            for j, pw in e.items():
                v = mp.mpf(pw) * yv[j] ** (pw - 1)
                for j2, pw2 in e.items():
                    if j2 != j:
                        v *= yv[j2] ** pw2
                D[r, j] = v
        return D

    def f(yv):
        mm = mono(yv)
        return S * mp.matrix([k[r] * mm[r] for r in range(nr)])

    D = dmono(y)
    J = S * mp.matrix([[k[r] * D[r, j] for j in range(nv)] for r in range(nr)])
    W = mp.eye(nv) / (mp.mpf(dm.g) * h) - J
    K, F = [], None
    zero = mp.zeros(nv, 1)
    for i in range(dm.st):
        Yi = y + sum((dm.a(i, j) * K[j] for j in range(i)), zero) if i else y
        if dm.NewF[i]:
            F = f(Yi)
        K.append(mp.lu_solve(W, F + sum((dm.c(i, j) / h * K[j] for j in range(i)), zero)))
    return y + sum((dm.M[i] * K[i] for i in range(dm.st)), zero)


@pytest.mark.parametrize("mech", RODAS3)
def test_rodas3_derivatives_match_high_precision(hostsim, mech):
    """RODAS-3 (4 stages, C/h coefficients up to 4/h) amplifies round-off
    in the derivative with respect to a stiff rate constant beyond eps
    cond(W): on small_strato at h = 1e-3 its k = 4e7 column differs between
    tangent and adjoint by 2e-8 while cond(W) = 3.5e4.  So both are checked
    against the exact derivative instead: central differences of the step
    in 60-digit arithmetic (step 1e-25 relative), every column of
    d y_new / d y and d y_new / d k to 1e-7 of its largest entry."""
    import mpmath as mp

    from oracle.adjoint_ref import DenseModel

    lib = hostsim[mech]
    plan = load(mech)
    dm = DenseModel(mech)
    w, o, k, _ = _case(mech, 1)
    y = w.conc[plan.var_phys, 0]
    kc = k[:, 0]
    h = 1e-3
    tl_y, tl_k, ad_y, ad_k = _jacobians(lib, mech, y, kc, h)
    mp.mp.dps = 60
    ym = mp.matrix([mp.mpf(v) for v in y])
    km = [mp.mpf(v) for v in kc]
    for j in range(dm.nv + dm.nr):
        if j < dm.nv:
            d = mp.mpf(10) ** -25 * max(abs(ym[j]), mp.mpf(1))
            yp, yn = ym.copy(), ym.copy()
            yp[j] += d
            yn[j] -= d
            col = (_step_mp(dm, yp, km, h) - _step_mp(dm, yn, km, h)) / (2 * d)
            tl, ad = tl_y[:, j], ad_y[:, j]
        else:
            r = j - dm.nv
            d = mp.mpf(10) ** -25 * max(abs(km[r]), mp.mpf(1e-300))
            kp, kn = list(km), list(km)
            kp[r] += d
            kn[r] -= d
            col = (_step_mp(dm, ym, kp, h) - _step_mp(dm, ym, kn, h)) / (2 * d)
            tl, ad = tl_k[:, r], ad_k[:, r]
        col = np.array([float(c) for c in col])
        sc = max(np.abs(col).max(), 1e-300)
        assert np.abs(tl - col).max() <= 1e-7 * sc, (j, "tangent")
        assert np.abs(ad - col).max() <= 1e-7 * sc, (j, "adjoint")


@pytest.mark.parametrize("mech", MECHS)
def test_tangent_matches_dense_model(hostsim, mech):
    """d y_new / d y of the emitted tangent against the dense FP64 CPU model
    of the step (oracle/adjoint_ref.py: dense LU, its adjoint rows), to 1e-8
    of each column's largest entry."""
    from oracle.adjoint_ref import DenseModel

    lib = hostsim[mech]
    plan = load(mech)
    dm = DenseModel(mech)
    w, o, k, _ = _case(mech, 1)
    y = w.conc[plan.var_phys, 0]
    kc = k[:, 0]
    nv = plan.n_var
    h = 1e-2
    tl = np.zeros((nv, nv))
    for j in range(nv):
        e = np.zeros(nv)
        e[j] = 1.0
        tl[:, j] = _host_tlm(lib, y, kc, h, e, np.zeros(len(kc)))[0]
    _, tape = dm.forward(y, kc, [h])
    dense = np.zeros((nv, nv))
    for i in range(nv):
        e = np.zeros(nv)
        e[i] = 1.0
        dense[i, :] = dm.adjoint(kc, tape, e)[0]
    assert _column_error(tl, dense) <= 1e-8


@pytest.mark.parametrize("mech", MECHS + EXTRA + ["ts1"])
def test_tangent_taylor_test(hostsim, mech):
    """Taylor test of the emitted tangent through a whole accepted-step
    sequence (the oracle's 60 s integration, steps then frozen): for a
    direction (dy, dk) scaled by (y, k), the remainder
    |Y(y + e dy, k + e dk) - Y(y, k) - e T (dy, dk)| falls 4x when e halves
    (measured 3.98-4.17 down to e = 2e-5 on chapman, small_strato,
    saprc99_mini and SAPRC99; TS1, through its table-driven tangent, 4.000
    down to e = 2.5e-4, below which round-off dominates).  The reference
    checks its frozen-Jacobian tangent the same way
    (tests/python/test_taylor_test_tlm.py)."""
    lib = hostsim[mech]
    plan = load(mech)
    w, o, k, dk = _case(mech, 1)
    rep = o.integrate(w.conc.copy(), 60.0, k=k, dk=dk, temp=w.temp, rho=w.rho, rh=w.rh, param=w.param,
                      log_cap=4096)
    n = rep["log_n"][0]
    hs = rep["log_h"][:n, 0][rep["log_acc"][:n, 0].astype(bool)]
    assert len(hs) > 5
    y0, kc = w.conc[plan.var_phys, 0].copy(), k[:, 0].copy()
    rng = np.random.default_rng(1)
    dy0 = rng.uniform(-1.0, 1.0, len(y0)) * y0
    dk0 = rng.uniform(-1.0, 1.0, len(kc)) * kc
    zero_y, zero_k = np.zeros(len(y0)), np.zeros(len(kc))

    def run(y, kk, dy, dkk):
        for h in hs:
            dy, y, st = _host_tlm(lib, y, kk, h, dy, dkk)
            assert st == 0
        return y, dy

    Y, T = run(y0, kc, dy0, dk0)
    scale = np.abs(Y) + 1.0
    r = []
    # TS1 (cond(W) up to 1e10) reaches its round-off floor at larger e.
    e0 = 4e-3 if mech == "ts1" else 1e-3
    for e in (e0, e0 / 2, e0 / 4, e0 / 8):
        Ye, _ = run(y0 + e * dy0, kc + e * dk0, zero_y, zero_k)
        r.append(np.max(np.abs(Ye - Y - e * T) / scale))
    ratios = np.array(r[:-1]) / np.array(r[1:])
    assert np.all((ratios > 3.9) & (ratios < 4.1)), ratios


@pytest.mark.parametrize("mech", MECHS + EXTRA + ["ts1"])
def test_emitted_rate_constants_match_oracle(hostsim, mech):
    """The emitted rate_constants() (the code rate_constant_kernel runs),
    compiled for the host, against the oracle's rate constants on seeded
    cells: 1e-13 relative (glibc vs numpy exp/log/pow).  This pins the
    emitted expressions, their parameter-slot, fixed-species and
    environment arguments for every mechanism, TS1's 547 included."""
    lib = hostsim[mech]
    lib.hostsim_rate_constants.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                           C.c_double, C.c_void_p]
    n = 16
    w = workloads.make(mech, n)
    o = Oracle(mech)
    k_ref, _ = o.rate_constants(w.conc, w.temp, w.rho, w.rh, None, w.param)
    for c in range(n):
        conc = np.ascontiguousarray(w.conc[:, c])
        prm = np.ascontiguousarray(w.param[:, c]) if w.param.shape[0] else None
        k = np.zeros(k_ref.shape[0])
        lib.hostsim_rate_constants(conc.ctypes.data, None if prm is None else prm.ctypes.data, w.temp[c],
                                   w.rho[c], w.rh[c], 0.0, k.ctypes.data)
        np.testing.assert_allclose(k, k_ref[:, c], rtol=1e-13, atol=0)


@pytest.mark.parametrize("mech", MECHS + EXTRA)
def test_emitted_tendencies_and_jacobian_match_reference(hostsim, mech):
    """The emitted fun(), jac_w() and jac_fixed_columns() (what the GPU
    evaluation entries run), compiled for the host and fed the emitted rate
    constants, against the reference's own generated compute_rates /
    compute_jacobian built here (oracle/ref_build.py): F to 1e-13 of the
    cell's largest |F|, every nonzero J entry to 1e-11, and zeros wherever the
    reference writes none.  The two sum the mass-action terms in different
    orders."""
    from oracle import ref_build

    try:
        if mech in ref_build.MECHS:
            ref_build.build_if_available()
            ref = ref_build.load(mech)
        else:
            ref = ref_build.ensure(mech)
    except Exception as e:  # noqa: BLE001
        pytest.skip(f"reference build failed: {e}")
    if ref is None:
        pytest.skip("reference solver library not built")
    lib = hostsim[mech]
    lib.hostsim_rate_constants.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                           C.c_double, C.c_void_p]
    lib.hostsim_evaluate.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_void_p, C.c_void_p, C.c_void_p]
    n = 16
    w = workloads.make(mech, n)
    F0, J0 = ref.evaluate(w.conc, w.temp, w.rho, w.rh, w.param)
    ns, nr = F0.shape[0], len(load(mech).reactions)
    for c in range(n):
        conc = np.ascontiguousarray(w.conc[:, c])
        prm = np.ascontiguousarray(w.param[:, c]) if w.param.shape[0] else None
        pp = None if prm is None else prm.ctypes.data
        k = np.zeros(nr)
        lib.hostsim_rate_constants(conc.ctypes.data, pp, w.temp[c], w.rho[c], w.rh[c], 0.0, k.ctypes.data)
        F, J = np.zeros(ns), np.zeros(ns * ns)
        assert lib.hostsim_evaluate(conc.ctypes.data, pp, w.temp[c], w.rho[c], w.rh[c], 0.0, k.ctypes.data,
                                    F.ctypes.data, J.ctypes.data) == 0
        J = J.reshape(ns, ns).T                       # [row, col]
        assert np.abs(F - F0[:, c]).max() <= 1e-13 * max(np.abs(F0[:, c]).max(), 1e-300)
        nz = J0[:, :, c] != 0
        assert not np.any(J[~nz])
        assert (np.abs(J - J0[:, :, c])[nz] / np.abs(J0[:, :, c][nz])).max() < 1e-11


def test_ts1_table_evaluation_matches_reference_fixture(hostsim):
    """TS1's table-driven evaluation program (eval_step: the partials, W with
    1/(gamma h) = 0 and F, walked by one thread) with the emitted rate
    constants and fixed-species columns, against the reference's own
    generated TS1 compute_rates / compute_jacobian
    (tests/golden/ts1_reference_rates.json, at the inputs of its native TS1
    run, photolysis scaled by 1.0 and 1.05): F to 1e-13 of the largest |F|,
    every nonzero J entry to 1e-11, zeros where the reference writes none."""
    import json

    lib = hostsim["ts1"]
    lib.hostsim_rate_constants.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                           C.c_double, C.c_void_p]
    lib.hostsim_evaluate.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_void_p, C.c_void_p, C.c_void_p]
    here = Path(__file__).resolve().parent / "golden"
    g = json.loads((here / "ts1_kokkos_2x300.json").read_text())
    rates = json.loads((here / "ts1_reference_rates.json").read_text())
    conc = np.ascontiguousarray(g["initial"], dtype=np.float64)
    ns, nr = len(conc), len(load("ts1").reactions)
    for case in rates["cases"]:
        prm = np.array(g["parameters"], dtype=np.float64)
        prm[:g["photolysis_slots"]] *= case["photolysis_scale"]
        k = np.zeros(nr)
        lib.hostsim_rate_constants(conc.ctypes.data, prm.ctypes.data, g["temperature"], g["air_density"],
                                   g["rh"], 0.0, k.ctypes.data)
        F, J = np.zeros(ns), np.zeros(ns * ns)
        assert lib.hostsim_evaluate(conc.ctypes.data, prm.ctypes.data, g["temperature"], g["air_density"],
                                    g["rh"], 0.0, k.ctypes.data, F.ctypes.data, J.ctypes.data) == 0
        J = J.reshape(ns, ns).T                       # [row, col]
        F0 = np.array(case["F"])
        assert np.abs(F - F0).max() <= 1e-13 * np.abs(F0).max()
        J0 = np.zeros((ns, ns))
        for i, j, v in case["J"]:
            J0[i, j] = v
        nz = J0 != 0
        assert not np.any(J[~nz])
        assert (np.abs(J - J0)[nz] / np.abs(J0[nz])).max() < 1e-11

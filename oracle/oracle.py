"""CPU oracle wrapper (TEST INFRASTRUCTURE ONLY).

Loads a mechanism plan JSON, lays its tables out for ``mkpp_oracle.c`` and runs
the C restatement of the reference's per-cell Rosenbrock solve.  Only tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use this
module; the product library never imports it.

Rate constants are evaluated here with numpy from the rate-constant
expressions the plan exporter split off the reference's reaction fluxes
(``src/mkpp/lowering.py:167-432``), with the fixed-species concentrations,
temperature and air density of each cell.
"""

from __future__ import annotations

import ctypes as C
import json
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
LIB = BUILD / "libmkpp_oracle.so"
MECH_DIR = ROOT / "mkpp_gb300" / "mechanisms"
MAXST = 6


def build(force: bool = False) -> Path:
    src = HERE / "mkpp_oracle.c"
    if LIB.exists() and not force and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    cc = os.environ.get("CC", "gcc")
    subprocess.run([cc, "-O2", "-fopenmp", "-shared", "-fPIC", str(src), "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)


class _Plan(C.Structure):
    _fields_ = [
        ("ns", C.c_int), ("nr", C.c_int),
        ("fixed", _IP), ("perm", _IP),
        ("react_off", _IP), ("react_sp", _IP), ("react_pow", _IP),
        ("net_off", _IP), ("net_sp", _IP), ("net_c", _DP),
        ("dk_off", _IP), ("dk_sp", _IP),
        ("nj", C.c_int), ("jslot_of", _IP),
        ("nw", C.c_int), ("w_diag", _IP), ("w_jslot", _IP),
        ("nlu", C.c_int), ("nops", C.c_int),
        ("op_out", _IP), ("op_w", _IP), ("op_begin", _IP), ("op_end", _IP), ("op_diag", _IP),
        ("prod_l", _IP), ("prod_r", _IP),
        ("lower_off", _IP), ("lower_col", _IP), ("lower_slot", _IP),
        ("upper_off", _IP), ("upper_col", _IP), ("upper_slot", _IP),
        ("diag", _IP),
        ("stages", C.c_int), ("gamma", C.c_double), ("elo", C.c_double),
        ("A", C.c_double * (MAXST * MAXST)), ("C", C.c_double * (MAXST * MAXST)),
        ("M", C.c_double * MAXST), ("E", C.c_double * MAXST), ("newf", C.c_int * MAXST),
        ("atol", _DP), ("rtol", _DP),
    ]


def _i(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32).reshape(-1) if len(a) else np.zeros(1, np.int32))


def _d(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1) if len(a) else np.zeros(1, np.float64))


def _ptr(a, t):
    return a.ctypes.data_as(t)


class Oracle:
    """The C restatement bound to one mechanism plan."""

    def __init__(self, mech: str | dict, tableau: dict | None = None):
        raw = mech if isinstance(mech, dict) else json.loads((MECH_DIR / f"{mech}.plan.json").read_text())
        self.raw = raw
        self.name = raw["name"]
        self.lib = C.CDLL(str(build()))
        self.lib.mkpp_oracle_integrate.restype = C.c_int
        self.lib.mkpp_oracle_eval.restype = C.c_int
        ns = len(raw["species"])
        nr = len(raw["reactions"])
        self.ns, self.nr = ns, nr
        comp = raw["compact"]
        keep = []

        def arr(x, kind="i"):
            a = _i(x) if kind == "i" else _d(x)
            keep.append(a)
            return a

        react_off, react_sp, react_pow = [0], [], []
        net_off, net_sp, net_c = [0], [], []
        dk_off, dk_sp = [0], []
        self.dk_exprs = []
        for r in raw["reactions"]:
            for s, pw in r["reactants"]:
                react_sp.append(s)
                react_pow.append(pw)
            react_off.append(len(react_sp))
            for s, c in r["net"]:
                net_sp.append(s)
                net_c.append(c)
            net_off.append(len(net_sp))
            for f, e in r.get("dk_dfixed", []):
                dk_sp.append(f)
                self.dk_exprs.append(e)
            dk_off.append(len(dk_sp))
        jslot = -np.ones(ns * ns, dtype=np.int32)
        for slot, (i, j) in enumerate(raw["jacobian_entries"]):
            jslot[i * ns + j] = slot
        w_loc = comp["w_locations"]
        ops = np.asarray(comp["operations"], dtype=np.int32).reshape(-1, 5)
        prods = np.asarray(comp["products"], dtype=np.int32).reshape(-1, 2)
        low = np.asarray(comp["lower"], dtype=np.int32).reshape(-1, 2)
        up = np.asarray(comp["upper"], dtype=np.int32).reshape(-1, 2)
        tab = tableau or raw["tableau"]
        st = int(tab["stages"])
        p = _Plan()
        p.ns, p.nr = ns, nr
        p.fixed = _ptr(arr([int(x) for x in raw["fixed"]]), _IP)
        p.perm = _ptr(arr(raw["permutation"]), _IP)
        p.react_off = _ptr(arr(react_off), _IP)
        p.react_sp = _ptr(arr(react_sp), _IP)
        p.react_pow = _ptr(arr(react_pow), _IP)
        p.net_off = _ptr(arr(net_off), _IP)
        p.net_sp = _ptr(arr(net_sp), _IP)
        p.net_c = _ptr(arr(net_c, "d"), _DP)
        p.dk_off = _ptr(arr(dk_off), _IP)
        p.dk_sp = _ptr(arr(dk_sp), _IP)
        p.nj = len(raw["jacobian_entries"])
        p.jslot_of = _ptr(arr(jslot), _IP)
        p.nw = len(w_loc)
        p.w_diag = _ptr(arr([int(a == b) for a, b in w_loc]), _IP)
        p.w_jslot = _ptr(arr(comp["j_slot_of_w"]), _IP)
        p.nlu = len(comp["lu_locations"])
        p.nops = len(ops)
        for k_, col in zip(("op_out", "op_w", "op_begin", "op_end", "op_diag"), range(5)):
            setattr(p, k_, _ptr(arr(ops[:, col]), _IP))
        p.prod_l = _ptr(arr(prods[:, 0]), _IP)
        p.prod_r = _ptr(arr(prods[:, 1]), _IP)
        p.lower_off = _ptr(arr(comp["lower_offsets"]), _IP)
        p.lower_col = _ptr(arr(low[:, 0]), _IP)
        p.lower_slot = _ptr(arr(low[:, 1]), _IP)
        p.upper_off = _ptr(arr(comp["upper_offsets"]), _IP)
        p.upper_col = _ptr(arr(up[:, 0]), _IP)
        p.upper_slot = _ptr(arr(up[:, 1]), _IP)
        p.diag = _ptr(arr(comp["diagonals"]), _IP)
        p.stages = st
        p.gamma = float(tab["Gamma"][0])
        p.elo = float(tab["ELO"])
        for s_ in range(1, st):
            for j in range(s_):
                idx = s_ * (s_ - 1) // 2 + j
                p.A[s_ * MAXST + j] = tab["A"][idx]
                p.C[s_ * MAXST + j] = tab["C"][idx]
        for j in range(st):
            p.M[j] = tab["M"][j]
            p.E[j] = tab["E"][j]
            p.newf[j] = int(bool(tab["NewF"][j]))
        p.atol = _ptr(arr(raw["atol"], "d"), _DP)
        p.rtol = _ptr(arr(raw["rtol"], "d"), _DP)
        self._keep = keep
        self.plan = p
        self.ndk = len(dk_sp)
        self.seed = float(raw["initial_step_seed"])

    # ------------------------------------------------------------------
    def _env(self, conc, temp, rho, rh, clw, param):
        n = conc.shape[1]
        raw = self.raw
        if raw["runtime_environment"]:
            T = np.asarray(temp, dtype=np.float64)
            RHO = np.asarray(rho, dtype=np.float64)
        else:
            T = np.full(n, raw["environment_temperature"])
            RHO = np.full(n, raw["environment_air_density"])
        RH = np.full(n, 0.5) if rh is None else np.asarray(rh, dtype=np.float64)
        CLW = np.zeros(n) if clw is None else np.asarray(clw, dtype=np.float64)
        P = np.zeros((max(1, raw["num_rate_parameters"]), n)) if param is None else np.asarray(param, np.float64)
        return {
            "pow": np.power, "exp": np.exp, "log": np.log, "sqrt": np.sqrt, "fabs": np.abs,
            "M_LN10": math.log(10.0), "P": P, "FIX": conc, "T": T, "RHO": RHO, "RH": RH, "CLW": CLW,
        }

    def rate_constants(self, conc, temp=None, rho=None, rh=None, clw=None, param=None):
        """k[r][cell] and dk[e][cell] for (species x cells) LayoutLeft inputs."""
        conc = np.asarray(conc, dtype=np.float64)
        n = conc.shape[1]
        env = self._env(conc, temp, rho, rh, clw, param)
        with np.errstate(all="ignore"):
            k = np.empty((self.nr, n))
            for r, rr in enumerate(self.raw["reactions"]):
                k[r] = np.broadcast_to(eval(rr["k"], env), (n,))
            dk = np.empty((max(1, self.ndk), n))
            for e, ex in enumerate(self.dk_exprs):
                dk[e] = np.broadcast_to(eval(ex, env), (n,))
        return k, dk

    def integrate(self, conc, dt, steps=1, temp=None, rho=None, rh=None, clw=None, param=None,
                  seed=None, max_attempts=20000, nthreads=0, log_cap=0, replay=None, k=None, dk=None,
                  dt_carry=None):
        """Integrate in place a (species x cells) array; returns a dict of diagnostics.
        dt_carry: optional float64 [cells] array, in/out, for step-size
        carry-over across integrate() calls (0: start at dt * seed)."""
        conc = np.ascontiguousarray(conc, dtype=np.float64)
        ns, n = conc.shape
        assert ns == self.ns
        if k is None:
            k, dk = self.rate_constants(conc, temp, rho, rh, clw, param)
        k = np.ascontiguousarray(k, dtype=np.float64)
        dk = np.ascontiguousarray(dk, dtype=np.float64)
        status = np.zeros(n, np.int32)
        acc = np.zeros(n, np.int32)
        rej = np.zeros(n, np.int32)
        out = {"status": status, "accepted": acc, "rejected": rej}
        lh = la = ln = None
        if log_cap:
            lh = np.zeros((log_cap, n))
            la = np.zeros((log_cap, n), np.uint8)
            ln = np.zeros(n, np.int32)
            out.update(log_h=lh, log_acc=la, log_n=ln)
        if dt_carry is not None:
            assert dt_carry.dtype == np.float64 and dt_carry.shape == (n,) and dt_carry.flags.c_contiguous
        rh_ = ra_ = rn_ = None
        if replay is not None:
            rh_ = np.ascontiguousarray(replay[0], dtype=np.float64)
            ra_ = np.ascontiguousarray(replay[1], dtype=np.uint8)
            rn_ = np.ascontiguousarray(replay[2], dtype=np.int32)
        vp = C.c_void_p

        def p(a):
            return vp(a.ctypes.data) if a is not None else None

        fails = self.lib.mkpp_oracle_integrate(
            C.byref(self.plan), C.c_int(n), p(conc), p(k), p(dk), C.c_int(self.ndk), C.c_double(dt),
            C.c_int(steps), C.c_double(self.seed if seed is None else seed), C.c_int(max_attempts),
            C.c_int(nthreads), p(status), p(acc), p(rej), p(lh), p(la), p(ln), C.c_int(log_cap),
            p(rh_), p(ra_), p(rn_), p(dt_carry))
        out["failures"] = fails
        out["conc"] = conc
        return out

    def evaluate(self, conc, temp=None, rho=None, rh=None, clw=None, param=None):
        """(F [ns][cells], J [nj][cells]) at the given states."""
        conc = np.ascontiguousarray(conc, dtype=np.float64)
        n = conc.shape[1]
        k, dk = self.rate_constants(conc, temp, rho, rh, clw, param)
        F = np.zeros((self.ns, n))
        J = np.zeros((max(1, len(self.raw["jacobian_entries"])), n))
        vp = C.c_void_p
        rc = self.lib.mkpp_oracle_eval(C.byref(self.plan), C.c_int(n), vp(conc.ctypes.data), vp(k.ctypes.data),
                                       vp(dk.ctypes.data), C.c_int(self.ndk), vp(F.ctypes.data), vp(J.ctypes.data))
        assert rc == 0
        return F, J

    def dense_jacobian(self, J):
        """Compact J slots -> dense (ns, ns, cells) with J[i, j, c]."""
        n = J.shape[1]
        D = np.zeros((self.ns, self.ns, n))
        for slot, (i, j) in enumerate(self.raw["jacobian_entries"]):
            D[i, j] = J[slot]
        return D

"""Pin the CPU oracle to the reference's own published outputs and tests."""
import copy
import json
from pathlib import Path

import numpy as np
import pytest

from oracle.oracle import Oracle
from mkpp_gb300.emitter.plan import load_raw

GOLD = Path(__file__).resolve().parent / "golden"


def _with_tol(mech, rtol, atol):
    raw = copy.deepcopy(load_raw(mech))
    raw["rtol"] = [rtol] * len(raw["species"])
    raw["atol"] = [atol] * len(raw["species"])
    return raw


def test_chapman_native_kokkos_run():
    """1 cell, 10 x 60 s, shipped tolerances: final state of the reference's native run."""
    g = json.loads((GOLD / "chapman_kokkos_10x60.json").read_text())
    o = Oracle(_with_tol("chapman", g["tolerances"]["rtol"], g["tolerances"]["atol"]))
    names = o.raw["species"]
    conc = np.array([[g["initial"][s]] for s in names])
    out = o.integrate(conc, g["dt"], steps=g["steps"], param=np.array(g["jvals"])[:, None])
    got = out["conc"][:, 0]
    want = np.array([g["final"][s] for s in names])
    np.testing.assert_allclose(got, want, rtol=1e-14, atol=0)


@pytest.mark.parametrize("rtol,atol", [(1e-6, 1e-3), (1e-3, 1.0)])
def test_chapman_scipy_radau_golden(rtol, atol):
    """tests/integration/e2e_validation/test_scipy_validation.cpp gate: |d| <= 1 + 1e-4 |ref|."""
    g = json.loads((GOLD / "chapman_scipy_reference.json").read_text())
    o = Oracle(_with_tol("chapman", rtol, atol))
    conc = np.array(g["initial_conditions"], dtype=float)[:, None]
    out = o.integrate(conc, g["time_span"][1], param=np.array(g["jvals"])[:, None])
    got = out["conc"][:, 0]
    want = np.array(g["expected_final"])
    assert np.all(np.abs(got - want) <= g["gate"]["atol"] + g["gate"]["rtol"] * np.abs(want))


def test_factorization_known_answer():
    """13-slot Chapman W -> factorize_plan -> solve_plan, residual <= 1e-12."""
    g = json.loads((GOLD / "chapman_factorization_kat.json").read_text())
    raw = load_raw("chapman")
    comp = raw["compact"]
    w = g["w"]
    lu = [0.0] * len(comp["lu_locations"])
    prods = comp["products"]
    for out, wi, b, e, dg in comp["operations"]:
        v = w[wi] if wi >= 0 else 0.0
        for q in range(b, e):
            v -= lu[prods[q][0]] * lu[prods[q][1]]
        lu[out] = v / lu[dg] if dg >= 0 else v
    n = 4
    work = [0.0] * n
    x = [0.0] * n
    lo, up = comp["lower"], comp["upper"]
    for r in range(n):
        work[r] = g["rhs"][r]
        for e in range(comp["lower_offsets"][r], comp["lower_offsets"][r + 1]):
            work[r] -= lu[lo[e][1]] * work[lo[e][0]]
    for r in range(n - 1, -1, -1):
        x[r] = work[r]
        for e in range(comp["upper_offsets"][r], comp["upper_offsets"][r + 1]):
            x[r] -= lu[up[e][1]] * x[up[e][0]]
        x[r] /= lu[comp["diagonals"][r]]
    A = np.array(g["dense_logical"]).reshape(n, n)
    assert np.max(np.abs(A @ np.array(x) - np.array(g["rhs"]))) <= g["residual_tol"]


def test_oracle_replay_reproduces_free_run():
    """Replaying the oracle's own step log reproduces its free run bit for bit."""
    from mkpp_gb300 import workloads

    w = workloads.make("small_strato", 256)
    o = Oracle("small_strato")
    a = o.integrate(w.conc.copy(), w.dt, param=w.param, log_cap=512)
    b = o.integrate(w.conc.copy(), w.dt, param=w.param, replay=(a["log_h"], a["log_acc"], a["log_n"]))
    assert np.array_equal(a["conc"], b["conc"])


def test_oracle_flags_non_finite_cell():
    """A NaN in one cell's state is reported for that cell only (test_e2e_batched.cpp)."""
    from mkpp_gb300 import workloads

    w = workloads.make("chapman", 16)
    conc = w.conc.copy()
    conc[0, 5] = np.nan
    out = Oracle("chapman").integrate(conc, w.dt, param=w.param)
    assert out["status"][5] == 2
    assert np.all(np.delete(out["status"], 5) == 0)


def test_chapman_shipped_plan_reproduces_native_run():
    """The chapman_shipped plan (Chapman exported at the shipped tolerances,
    the plan of the GPU library that tests/test_gpu_golden.py runs) gives the
    reference's native-run final state through the oracle, to 1e-14."""
    g = json.loads((GOLD / "chapman_kokkos_10x60.json").read_text())
    o = Oracle("chapman_shipped")
    names = o.raw["species"]
    conc = np.array([[g["initial"][s]] for s in names])
    out = o.integrate(conc, g["dt"], steps=g["steps"], param=np.array(g["jvals"])[:, None])
    want = np.array([g["final"][s] for s in names])
    np.testing.assert_allclose(out["conc"][:, 0], want, rtol=1e-14, atol=0)

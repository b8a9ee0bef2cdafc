"""Static warp schedules of the cooperative LU and solves (CPU).

* The LU program factors W (L U = W with unit L) and the solve program solves
  W x = b, run sequentially in program order.
* Executed step by step (all lanes of a step read, then write), the schedule
  leaves every slot bit-identical to program order: any missing hazard edge
  changes some value on random data.
* Each step holds at most 32 operations with distinct outputs, and the
  header's tables are the encoded schedules.
"""

import re

import numpy as np
import pytest

from mkpp_gb300.emitter import warp_schedule as ws
from mkpp_gb300.emitter.cuda_emitter import GEN_DIR
from mkpp_gb300.emitter.plan import load

MECHS = ["chapman", "small_strato", "saprc99"]


def _apply(S, op, base):
    kind, out, a, b = op
    o = out if base is None else base + out
    bb = b if (base is None or kind != ws.FMA) else base + b
    if kind == ws.FMA:
        return o, S[o] - S[a] * S[bb]
    if kind == ws.MUL:
        return o, S[o] * S[bb]
    return o, 1.0 / S[o]


def _sequential(prog, S, base=None):
    S = S.copy()
    for op in prog:
        o, v = _apply(S, op, base)
        S[o] = v
    return S


def _stepped(prog, steps, S, base=None):
    S = S.copy()
    for batch in steps:
        upd = [_apply(S, prog[i], base) for i in batch]
        for o, v in upd:
            S[o] = v
    return S


def _store(plan, rng):
    """LU slots holding a diagonally dominant W on the pattern, fill-in zero."""
    n = plan.n_var
    nslot = max(plan.lu_index.values()) + 1
    S = np.zeros(nslot + 2 * n)
    W = np.zeros((n, n))
    for (r, c), sl in plan.lu_index.items():
        if (r, c) in plan.w_slots:
            W[r, c] = rng.uniform(-1.0, 1.0)
    W += np.diag(np.abs(W).sum(axis=1) + 1.0)
    for (r, c), sl in plan.lu_index.items():
        S[sl] = W[r, c]
    for sl in ws.lu_zero_slots(plan):
        S[sl] = 0.0
    return S, W, nslot


@pytest.mark.parametrize("mech", MECHS)
def test_programs_factor_and_solve(mech):
    plan = load(mech)
    n = plan.n_var
    rng = np.random.default_rng(3)
    S, W, nslot = _store(plan, rng)
    S = _sequential(ws.lu_program(plan), S)
    L, U = np.eye(n), np.zeros((n, n))
    for (r, c), sl in plan.lu_index.items():
        if r > c:
            L[r, c] = S[sl]
        elif r < c:
            U[r, c] = S[sl]
    for i, sl in enumerate(plan.diag):
        U[i, i] = 1.0 / S[sl]
    np.testing.assert_allclose(L @ U, W, rtol=0, atol=1e-12 * np.abs(W).max())
    b = rng.uniform(-1.0, 1.0, n)
    S[nslot:nslot + n] = b
    x = _sequential(ws.solve_program(plan), S, base=nslot)[nslot:nslot + n]
    np.testing.assert_allclose(W @ x, b, rtol=0, atol=1e-12)


@pytest.mark.parametrize("mech", MECHS)
def test_schedules_are_bit_identical_to_program_order(mech):
    plan = load(mech)
    rng = np.random.default_rng(7)
    lu = ws.lu_program(plan)
    sv = ws.solve_program(plan)
    for prog, rel in ((lu, False), (sv, True)):
        steps = ws.schedule(prog, relative=rel)
        assert sorted(i for s in steps for i in s) == list(range(len(prog)))
        for batch in steps:
            assert len(batch) <= ws.LANES
            assert len({prog[i][1] for i in batch}) == len(batch)
        for trial in range(3):
            S, _, nslot = _store(plan, rng)
            S[nslot:] = rng.uniform(-1.0, 1.0, S.size - nslot)
            base = nslot if rel else None
            assert np.array_equal(_sequential(prog, S, base), _stepped(prog, steps, S, base))


def test_saprc99_schedule_fills_the_warp():
    plan = load("saprc99")
    lu = ws.lu_program(plan)
    steps = ws.schedule(lu)
    # 10485 operations, critical path 132: the LU keeps ~31 of 32 lanes busy.
    assert len(lu) / len(steps) > 30


@pytest.mark.parametrize("mech", MECHS)
def test_header_tables_are_the_schedules(mech):
    plan = load(mech)
    text = (GEN_DIR / f"{mech}.cuh").read_text()
    for name, prog, rel in (("lu_fs", ws.lu_program(plan), False), ("sv_fs", ws.solve_program(plan), True)):
        m = re.search(r"unsigned long long %s\[(\d+)\] = \{(.*?)\};" % name, text, re.S)
        assert m, name
        words = [int(w, 16) for w in re.findall(r"0x([0-9a-f]+)ull", m.group(2))]
        assert words == ws.encode(prog, ws.schedule(prog, relative=rel))
        for w in words[:64]:
            kind, out, a, b = ws.decode(w)
            assert w == (out | (a << 16) | (b << 32) | (kind << 48))

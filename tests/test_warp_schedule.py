"""Static warp schedules of the cooperative attempt (CPU).

* The LU program factors W (L U = W, unit L) and the solve program solves
  W x = b, run in program order.
* The three stage programs of the cooperative attempt compute the
  Rosenbrock stages of a dense CPU model (oracle/adjoint_ref.py): the LU
  reproduces W, F matches at every stage state, and each K_i solves its
  stage system to round-off.
* Executed step by step (all lanes of a step read, then write), each
  schedule leaves every slot bit-identical to program order: a missing
  hazard edge changes some value on random data.
* Each step holds at most 32 operations with distinct outputs, and the
  header's table is the encoded schedules.

The arithmetic here is plain float64 (a*b + c, not fused): it checks the
order of operations and the data flow.  Bit-identity with the per-thread
kernel, whose fma() fuse, is checked on the GPU.
"""

import re

import numpy as np
import pytest

from mkpp_gb300.emitter import cuda_emitter
from mkpp_gb300.emitter import warp_schedule as ws
from mkpp_gb300.emitter.cuda_emitter import GEN_DIR
from mkpp_gb300.emitter.plan import load

MECHS = ["chapman", "small_strato", "saprc99"]


def _apply(S, op):
    kind, out, a, b, c, neg = op
    if kind == ws.RCP:
        return out, 1.0 / S[out]
    x = -S[a] if neg else S[a]
    return out, x * S[b] + S[c]


def _sequential(ops, S):
    S = S.copy()
    for op in ops:
        o, v = _apply(S, op)
        S[o] = v
    return S


def _stepped(ops, steps, S):
    S = S.copy()
    for batch in steps:
        upd = [_apply(S, ops[i]) for i in batch]
        for o, v in upd:
            S[o] = v
    return S


def _lu_store(plan, rng, extra):
    """Slots [LU | b | x | -0, +0, 1] with a diagonally dominant W on the
    pattern and the fill-in zero."""
    n = plan.n_var
    nslot = max(plan.lu_index.values()) + 1
    S = np.zeros(nslot + extra)
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


def _lu_solve_programs(plan, nslot):
    n = plan.n_var
    zn, zp, one = nslot + n, nslot + n + 1, nslot + n + 2
    lu = ws.Program(zn, zp, one, lit=None)
    lu.lu(plan)
    sv = ws.Program(zn, zp, one, lit=None)
    sv.solve(plan, nslot)
    return lu.ops, sv.ops, (zn, zp, one)


@pytest.mark.parametrize("mech", MECHS)
def test_lu_and_solve_programs(mech):
    plan = load(mech)
    n = plan.n_var
    rng = np.random.default_rng(3)
    S, W, nslot = _lu_store(plan, rng, n + 3)
    lu, sv, (zn, zp, one) = _lu_solve_programs(plan, nslot)
    S[zn], S[zp], S[one] = -0.0, 0.0, 1.0
    S = _sequential(lu, S)
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
    x = _sequential(sv, S)[nslot:nslot + n]
    np.testing.assert_allclose(W @ x, b, rtol=0, atol=1e-12)


def _coop(mech):
    plan = load(mech)
    cuda_emitter.emit_mechanism(plan)
    return plan, plan._coop_programs


def _stage_store(plan, info, y, k, h, gamma):
    S = np.zeros(info["slots"])
    nv = plan.n_var
    S[info["Y"]:info["Y"] + nv] = y
    S[info["KT"]:info["KT"] + len(k)] = k
    CB = info["CB"]
    S[CB:CB + 4] = (-0.0, 0.0, 1.0, 1.0 / (gamma * h))
    for (st, j), slot in info["cterm_slot"].items():
        S[slot] = info["C"][(st - 1) * (st - 2) // 2 + j - 1] / h
    for v, slot in info["literals"].items():
        S[slot] = v
    return S


@pytest.mark.parametrize("mech", MECHS)
def test_stage_programs_give_the_rosenbrock_stages(mech):
    """Stage by stage, without depending on the conditioning of W (up to
    5e9 here): the LU reproduces W = I/(gamma h) - J, F is the dense model's
    F at the stage state built from the program's own K_j, and each K_i
    solves W K_i = F_i + sum_j c_ij/h K_j to round-off."""
    from oracle.adjoint_ref import DenseModel
    from oracle.oracle import Oracle

    from mkpp_gb300 import workloads

    plan, (progs, sched, info) = _coop(mech)
    dm = DenseModel(mech)
    w = workloads.make(mech, 4)
    k_all, _ = Oracle(mech).rate_constants(w.conc, w.temp, w.rho, w.rh, None, w.param)
    nv = plan.n_var
    K0, FS = info["K0"], info["FS"]
    for c in range(4):
        y = w.conc[plan.var_phys, c]
        k = k_all[:, c]
        h = 10.0
        W = np.eye(nv) / (dm.g * h) - dm.J(y, k)
        S = _stage_store(plan, info, y, k, h, dm.g)
        Ks = []
        for i, ops in enumerate(progs):
            S = _sequential(ops, S)
            if i == 0:
                L, U = np.eye(nv), np.zeros((nv, nv))
                for (r, cc), sl in plan.lu_index.items():
                    if r > cc:
                        L[r, cc] = S[sl]
                    elif r < cc:
                        U[r, cc] = S[sl]
                for j, sl in enumerate(plan.diag):
                    U[j, j] = 1.0 / S[sl]
                np.testing.assert_allclose(L @ U, W, rtol=0, atol=1e-13 * np.abs(W).max())
            Yi = y + sum(dm.a(i, j) * Ks[j] for j in range(i)) if i else y
            F = S[FS:FS + nv]
            if dm.NewF[i]:
                Fd = dm.f(Yi, k)
                np.testing.assert_allclose(F, Fd, rtol=0, atol=1e-13 * max(np.abs(Fd).max(), 1e-300))
            Ki = S[K0 + i * nv:K0 + (i + 1) * nv].copy()
            rhs = F + sum(dm.c(i, j) / h * Ks[j] for j in range(i))
            scale = np.abs(W) @ np.abs(Ki) + np.abs(rhs)
            assert np.all(np.abs(W @ Ki - rhs) <= 1e-12 * scale.max())
            Ks.append(Ki)


@pytest.mark.parametrize("mech", MECHS)
def test_schedules_are_bit_identical_to_program_order(mech):
    plan, (progs, sched, info) = _coop(mech)
    rng = np.random.default_rng(7)
    S0, _, nslot = _lu_store(plan, rng, plan.n_var + 3)
    lu, sv, (zn, zp, one) = _lu_solve_programs(plan, nslot)
    S0[zn], S0[zp], S0[one] = -0.0, 0.0, 1.0
    S0[nslot:nslot + plan.n_var] = rng.uniform(-1.0, 1.0, plan.n_var)
    cases = [(lu, S0), (sv, S0)]
    for ops in progs:
        S = rng.uniform(0.5, 1.5, info["slots"])
        S[info["CB"]:info["CB"] + 3] = (-0.0, 0.0, 1.0)
        cases.append((ops, S))
    for ops, S in cases:
        steps = ws.schedule(ops)
        assert sorted(i for s in steps for i in s) == list(range(len(ops)))
        for batch in steps:
            assert len(batch) <= ws.LANES
            assert len({ops[i][1] for i in batch}) == len(batch)
        assert np.array_equal(_sequential(ops, S), _stepped(ops, steps, S))


def test_saprc99_lu_schedule_fills_the_warp():
    plan = load("saprc99")
    lu, _, _ = _lu_solve_programs(plan, max(plan.lu_index.values()) + 1)
    steps = ws.schedule(lu)
    # 10485 operations, critical path 132: the LU keeps ~31 of 32 lanes busy.
    assert len(lu) / len(steps) > 30


@pytest.mark.parametrize("mech", MECHS)
def test_header_table_is_the_schedules(mech):
    plan, (progs, sched, info) = _coop(mech)
    text = (GEN_DIR / f"{mech}.cuh").read_text()
    m = re.search(r"unsigned long long sched\[(\d+)\] = \{(.*?)\};", text, re.S)
    assert m
    words = [int(w, 16) for w in re.findall(r"0x([0-9a-f]+)ull", m.group(2))]
    expect = []
    for ops, st in zip(progs, sched):
        expect += ws.encode(ops, st)
    assert words == expect
    for wd in words[:256]:
        kind, out, a, b, c, neg = ws.decode(wd)
        if kind:
            assert ws.encode([(kind, out, a, b, c, neg)], [[0]])[0] == wd
    m = re.search(r"stage_step\[\d+\] = \{([^}]*)\}", text)
    offs = [int(x) for x in m.group(1).split(",")]
    assert offs == list(np.cumsum([0] + [len(s) for s in sched]))

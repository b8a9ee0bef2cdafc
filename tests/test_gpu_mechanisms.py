"""Further shipped mechanisms on the GPU: saprc99_mini (17 species, 13 reactions).

The same kernels and checks as the SAPRC99 parity tests, on a mechanism the
reference ships without a benchmark configuration:
* rate constants against the oracle, 1e-13 relative;
* forced step sequence (the oracle replays the GPU's attempted step sizes and
  accept flags): per species 1e-9 (|oracle| + atol), with the one shipped
  Troe rate of ~1e33 1/s (reaction 7) moderated to 1e3 as for SAPRC99;
* cells parked for the warp-cooperative kernel end bit-identical to cells
  that stay on one lane;
* heterogeneous cells (the reference's tests/native/heterogeneous_cells.cpp,
  here on chapman and saprc99_mini): each cell of a three-cell batch with
  different temperature, pressure, density, state and forcing gets the same
  tendencies and integrated state through the C ABI as when it is solved
  alone (exactly; the reference allows 1e-10), and a non-positive
  temperature is rejected with MKPP_ERROR_INVALID_ARGUMENT.
On the CPU the oracle matches the reference's own generated solver for this
mechanism (tests/test_oracle_reference.py) and the emitted code matches the
oracle's forced step (tests/test_emitted_host.py).
"""
import numpy as np
import pytest

from mkpp_gb300 import workloads
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

MECH = "saprc99_mini"
EXTREME = (7,)
CELLS = 256


@pytest.fixture(scope="module")
def lib():
    from mkpp_gb300 import build

    return build.build((MECH,))[0]


def _setup():
    import torch

    from mkpp_gb300.api import DeviceSolver

    w = workloads.make(MECH, CELLS)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return w, DeviceSolver(MECH), Oracle(MECH), d


def test_rate_constants(lib):
    w, s, o, d = _setup()
    k_gpu, status = s.rate_constants(d(w.conc), d(w.temp), d(w.rho), d(w.rh), None, d(w.param))
    k_ref, _ = o.rate_constants(w.conc, w.temp, w.rho, w.rh, None, w.param)
    np.testing.assert_allclose(k_gpu.cpu().numpy(), k_ref, rtol=1e-13, atol=0)
    assert int(status.sum()) == 0


def test_forced_step_sequence_parity(lib):
    import torch

    w, s, o, d = _setup()
    conc = d(w.conc)
    ktab, _ = s.rate_constants(conc, d(w.temp), d(w.rho), d(w.rh), None, d(w.param))
    for r in EXTREME:
        ktab[r] = torch.clamp(ktab[r], max=1e3)
    _, dk = o.rate_constants(w.conc, w.temp, w.rho, w.rh, None, w.param)
    log = s.integrate_logged(conc, ktab, w.dt, log_cap=8192)
    torch.cuda.synchronize()
    ln = log["log_n"].cpu().numpy()
    ok = (log["status"].cpu().numpy() == 0) & (ln < 8192)
    rep = o.integrate(w.conc.copy(), w.dt, k=ktab.cpu().numpy(), dk=dk, temp=w.temp, rho=w.rho, rh=w.rh,
                      param=w.param, replay=(log["log_h"].cpu().numpy(), log["log_acc"].cpu().numpy(), ln))
    ok &= rep["status"] == 0
    assert ok.mean() > 0.9
    got, ref = conc.cpu().numpy()[:, ok], rep["conc"][:, ok]
    atol = np.array(o.raw["atol"])[:, None]
    assert (np.abs(got - ref) / (np.abs(ref) + atol)).max() <= 1e-9


def test_cooperative_handoff_is_bit_identical(lib):
    import torch

    w, s, o, d = _setup()
    outs = []
    try:
        for defer in (0, 7):
            s.set_tuning(defer_after=defer)
            conc = d(w.conc)
            st, acc, rej = s.integrate(conc, w.dt, temp=d(w.temp), rho=d(w.rho), rh=d(w.rh), param=d(w.param),
                                       mode="persistent")
            torch.cuda.synchronize()
            outs.append((conc.cpu().numpy(), st.cpu().numpy(), acc.cpu().numpy(), rej.cpu().numpy()))
    finally:
        s.set_tuning(defer_after=0)
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("mech", ["chapman", MECH])
def test_heterogeneous_batch_equals_single_cells(lib, built_libs, mech):
    from mkpp_gb300.api import MechanismContext, MkppError

    n = 3
    w = workloads.make(mech, n)
    temp = np.array([280.0, 300.0, 320.0])
    pressure = np.array([9.0e4, 9.5e4, 1.0e5])
    rho = w.rho.copy()
    param = np.ascontiguousarray(w.param * (1.0 + np.arange(n))[None, :])

    def solve(conc, t, p, r, prm):
        ctx = MechanismContext(mech, conc.shape[1])
        try:
            ctx.set_state(conc, t, p, r)
            ctx.set_rate_parameters(prm)
            rates = ctx.evaluate_rates()
            ctx.integrate(w.dt)
            return rates
        finally:
            ctx.close()

    batch = np.ascontiguousarray(w.conc.copy())
    rates = solve(batch, temp.copy(), pressure.copy(), rho.copy(), param)
    for c in range(n):
        one = np.ascontiguousarray(w.conc[:, c:c + 1].copy())
        r1 = solve(one, temp[c:c + 1].copy(), pressure[c:c + 1].copy(), rho[c:c + 1].copy(),
                   np.ascontiguousarray(param[:, c:c + 1]))
        assert np.array_equal(r1[:, 0], rates[:, c])
        assert np.array_equal(one[:, 0], batch[:, c])
    # As the reference does: bind valid meteorology, then zero a temperature
    # in the bound array before integrating.
    t_bound = temp.copy()
    ctx = MechanismContext(mech, n)
    try:
        ctx.set_state(np.ascontiguousarray(w.conc.copy()), t_bound, pressure.copy(), rho.copy())
        ctx.set_rate_parameters(param)
        t_bound[0] = 0.0
        with pytest.raises(MkppError) as e:
            ctx.integrate(w.dt)
        assert e.value.code == -103
    finally:
        ctx.close()


@pytest.mark.parametrize("mech", ["chapman", MECH])
def test_jacobian_vector_products(lib, built_libs, mech):
    """mkpp_evaluate_jacobian_vector / _transpose_vector (the per-cell J delta
    of the reference's compute_tlm and J^T lambda of compute_adjoint) equal
    the dense Jacobian of mkpp_evaluate_jacobian applied on the host, to
    1e-13 of the sum of the absolute terms (the summation orders differ)."""
    from mkpp_gb300.api import MechanismContext

    n = 16
    w = workloads.make(mech, n)
    rng = np.random.default_rng(4)
    v = np.ascontiguousarray(rng.uniform(-1.0, 1.0, w.conc.shape))
    ctx = MechanismContext(mech, n)
    try:
        ctx.set_state(np.ascontiguousarray(w.conc), w.temp.copy(), w.pressure.copy(), w.rho.copy())
        ctx.set_aerosol(relative_humidity=w.rh.copy())
        ctx.set_rate_parameters(np.ascontiguousarray(w.param))
        J = np.transpose(ctx.evaluate_jacobian(), (2, 1, 0))     # [cell, row, col]
        jv = ctx.evaluate_jacobian_vector(v)
        jtv = ctx.evaluate_jacobian_vector(v, transpose=True)
    finally:
        ctx.close()
    vc = v.T                                                      # [cell, species]
    ref = np.einsum("cij,cj->ic", J, vc)
    ref_t = np.einsum("cji,cj->ic", J, vc)
    assert np.all(np.abs(jv - ref) <= 1e-13 * np.einsum("cij,cj->ic", np.abs(J), np.abs(vc)) + 1e-300)
    assert np.all(np.abs(jtv - ref_t) <= 1e-13 * np.einsum("cji,cj->ic", np.abs(J), np.abs(vc)) + 1e-300)


def test_initial_step_seed_is_honoured(built_libs):
    """mkpp_set_initial_step_seed (the reference's SolverKernels::
    initial_step_seed member, integrate.j2:42; its test_initial_step_seed.py
    checks the plumbing): a larger seed changes the attempt counts, and the
    result agrees with the oracle run at the same seed within the
    free-running bound (10 (rtol |o| + atol))."""
    from mkpp_gb300.api import MechanismContext

    n = 64
    w = workloads.make("chapman", n)
    o = Oracle("chapman")
    out = {}
    for seed in (None, 1e-3):
        host = np.ascontiguousarray(w.conc.copy())
        ctx = MechanismContext("chapman", n)
        try:
            if seed is not None:
                ctx.set_initial_step_seed(seed)
            ctx.set_state(host, w.temp.copy(), w.pressure.copy(), w.rho.copy())
            ctx.set_rate_parameters(np.ascontiguousarray(w.param))
            ctx.integrate(w.dt)
            st, acc, rej = ctx.cell_stats()
        finally:
            ctx.close()
        out[seed] = (host, acc + rej)
    assert not np.array_equal(out[None][1], out[1e-3][1])
    ref = o.integrate(w.conc.copy(), w.dt, param=w.param, seed=1e-3)
    tol = np.array(o.raw["rtol"])[:, None] * np.abs(ref["conc"]) + np.array(o.raw["atol"])[:, None]
    assert np.all(np.abs(out[1e-3][0] - ref["conc"]) <= 10 * tol)

"""Step-size carry-over across integrate() calls (mkpp_gpu_integrate_carry,
mkpp_set_dt_carryover), an option off by default.

The reference restarts every integrate() at dt * initial_step_seed and lists
carried step estimates as future work (SCALING_OPTIMIZATION_REPORT.md:27-29).
With carry-over each call starts at the step size the previous call ended
with, which changes the step sequence (results differ from the default
within the tolerances), so parity is against the oracle run with the same
option (oracle/mkpp_oracle.c, dt_carry):
* the window form (one persistent launch over all host steps), the same
  window parked on the warp-cooperative kernel, one launch per host step
  with the carried step sizes handed back in, the plain form and the host C
  ABI with mkpp_set_dt_carryover all end bit for bit alike, carried step
  sizes included;
* against the oracle with carry-over, free-running: cells whose per-call
  accepted/rejected counts agree end within rtol |oracle| + atol, all
  within 10x that, and their carried step sizes agree to 1e-9 relative;
* the later host steps need fewer attempts than without carry-over.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MECH = "small_strato"
CELLS = 512
STEPS = 4


def _setup():
    import torch

    from mkpp_gb300 import workloads
    from mkpp_gb300.api import DeviceSolver

    w = workloads.make(MECH, CELLS)
    s = DeviceSolver(MECH)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    conc0 = d(w.conc)
    nr = s.sizes.reactions
    ktab = torch.empty((STEPS, nr, CELLS), dtype=torch.float64, device="cuda")
    for h in range(STEPS):
        k, _ = s.rate_constants(conc0, d(w.temp), d(w.rho), d(w.rh), None, d(w.param_at(h)))
        ktab[h].copy_(k)
    return w, s, conc0, ktab


def _window(s, conc0, ktab, dt, mode="persistent"):
    import torch

    conc = conc0.clone()
    carry = torch.zeros(CELLS, dtype=torch.float64, device="cuda")
    st = torch.zeros(CELLS, dtype=torch.int32, device="cuda")
    acc, rej = torch.zeros_like(st), torch.zeros_like(st)
    s.integrate_k(conc, ktab, dt, steps=STEPS, k_step_stride=ktab[0].numel(), mode=mode, status=st, accepted=acc,
                  rejected=rej, dt_carry=carry)
    torch.cuda.synchronize()
    return conc, carry, st


def test_carry_forms_agree_bitwise(built_libs):
    import torch

    from mkpp_gb300.api import MechanismContext

    w, s, conc0, ktab = _setup()
    conc_w, carry_w, st_w = _window(s, conc0, ktab, w.dt)
    # One launch per host step, the carried step sizes handed back in.
    conc = conc0.clone()
    carry = torch.zeros(CELLS, dtype=torch.float64, device="cuda")
    st = torch.zeros(CELLS, dtype=torch.int32, device="cuda")
    for h in range(STEPS):
        s.integrate_k(conc, ktab[h].contiguous(), w.dt, status=st, dt_carry=carry)
    torch.cuda.synchronize()
    assert torch.equal(conc, conc_w) and torch.equal(carry, carry_w) and torch.equal(st, st_w)
    # Plain form, and the window with every cell parked after 3 attempts.
    conc_p, carry_p, _ = _window(s, conc0, ktab, w.dt, mode="plain")
    assert torch.equal(conc_p, conc_w) and torch.equal(carry_p, carry_w)
    s.set_tuning(defer_after=1)
    try:
        conc_c, carry_c, _ = _window(s, conc0, ktab, w.dt)
    finally:
        s.set_tuning(defer_after=3000)
    assert torch.equal(conc_c, conc_w) and torch.equal(carry_c, carry_w)
    # Host C ABI with mkpp_set_dt_carryover.
    host = np.ascontiguousarray(w.conc.copy())
    ctx = MechanismContext(MECH, CELLS)
    try:
        ctx.set_state(host, w.temp.copy(), w.pressure.copy(), w.rho.copy())
        ctx.set_aerosol(relative_humidity=w.rh.copy())
        ctx.set_dt_carryover(True)
        pars = [np.ascontiguousarray(w.param_at(h)) for h in range(STEPS)]
        for h in range(STEPS):
            ctx.set_rate_parameters(pars[h])
            ctx.integrate(w.dt)
    finally:
        ctx.close()
    assert np.array_equal(host, conc_w.cpu().numpy())


def test_carry_matches_oracle_with_carry(built_libs):
    import torch

    from oracle.oracle import Oracle

    w, s, conc0, ktab = _setup()
    o = Oracle(MECH)
    conc = conc0.clone()
    carry = torch.zeros(CELLS, dtype=torch.float64, device="cuda")
    st = torch.zeros(CELLS, dtype=torch.int32, device="cuda")
    oc, ocarry = w.conc.copy(), np.zeros(CELLS)
    same = np.ones(CELLS, bool)
    att_carry = att_plain = 0
    plain = conc0.clone()
    for h in range(STEPS):
        acc, rej = torch.zeros_like(st), torch.zeros_like(st)
        s.integrate_k(conc, ktab[h].contiguous(), w.dt, status=st, accepted=acc, rejected=rej, dt_carry=carry)
        pacc, prej = torch.zeros_like(st), torch.zeros_like(st)
        s.integrate_k(plain, ktab[h].contiguous(), w.dt, accepted=pacc, rejected=prej)
        torch.cuda.synchronize()
        r = o.integrate(oc, w.dt, temp=w.temp, rho=w.rho, rh=w.rh, param=w.param_at(h), dt_carry=ocarry)
        oc = r["conc"]
        same &= (acc.cpu().numpy() == r["accepted"]) & (rej.cpu().numpy() == r["rejected"])
        if h > 0:
            att_carry += int((acc + rej).sum())
            att_plain += int((pacc + prej).sum())
    ok = (st.cpu().numpy() == 0) & (r["status"] == 0)
    assert ok.mean() > 0.9 and same[ok].mean() > 0.8
    got = conc.cpu().numpy()
    tol = np.array(o.raw["rtol"])[:, None] * np.abs(oc) + np.array(o.raw["atol"])[:, None]
    err = np.abs(got - oc) / tol
    assert np.all(err[:, ok & same] <= 1.0)
    assert np.all(err[:, ok] <= 10.0)
    cg = carry.cpu().numpy()
    assert np.all(np.abs(cg - ocarry)[ok & same] <= 1e-9 * np.abs(ocarry)[ok & same])
    # The ramp from dt * seed is gone from the later host steps.
    assert att_carry < 0.6 * att_plain

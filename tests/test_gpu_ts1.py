"""TS1 (210 species, 547 reactions) on the GPU: the table-driven library.

TS1 is too large for unrolled device code (49299 LU multiply-adds), so its
per-thread attempt walks the cooperative kernel's stage programs
(TABLE_ATTEMPT).  On the CPU the same emitted code is bit-identical to the
programs and matches the oracle's forced step (tests/test_emitted_host.py).
Here:
* rate constants against the oracle, 1e-13 relative;
* forced step sequence: the GPU logs its attempted step sizes and accept
  flags, the oracle replays them; per species 1e-9 (|oracle| + atol) on the
  cells both finish.  Six rate constants of the shipped TS1 reach 1e29-1e41
  1/s (Troe k0 evaluated as A exp(+C/T)); as for SAPRC99 they are moderated
  to 1e3 so that the comparison measures the arithmetic rather than the
  conditioning.  With them moderated, the oracle against itself under a
  one-ulp change of every rate constant moves by at most 1e-11 on these
  cells (atol 1 molec/cm3 in TS1's mol/m3), so 1e-9 is a gate on the
  arithmetic;
* the evaluation entries, table-driven too (one sequential program per
  cell for the partials, W and F), against the oracle.
"""
import numpy as np
import pytest

from mkpp_gb300 import workloads
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

EXTREME = (375, 376, 383, 394, 397, 402)
CELLS = 32


@pytest.fixture(scope="module")
def ts1_lib():
    from mkpp_gb300 import build

    return build.build(("ts1",))[0]


def _setup(n=CELLS):
    import torch

    from mkpp_gb300.api import DeviceSolver

    w = workloads.make("ts1", n)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return w, DeviceSolver("ts1"), Oracle("ts1"), d


def test_ts1_rate_constants(ts1_lib):
    w, s, o, d = _setup()
    k_gpu, status = s.rate_constants(d(w.conc), d(w.temp), d(w.rho), d(w.rh), None, d(w.param))
    k_ref, _ = o.rate_constants(w.conc, w.temp, w.rho, w.rh, None, w.param)
    np.testing.assert_allclose(k_gpu.cpu().numpy(), k_ref, rtol=1e-13, atol=0)
    assert int(status.sum()) == 0


def test_ts1_forced_step_sequence_parity(ts1_lib):
    import torch

    w, s, o, d = _setup()
    conc = d(w.conc)
    ktab, _ = s.rate_constants(conc, d(w.temp), d(w.rho), d(w.rh), None, d(w.param))
    for r in EXTREME:
        ktab[r] = torch.clamp(ktab[r], max=1e3)
    _, dk = o.rate_constants(w.conc, w.temp, w.rho, w.rh, None, w.param)
    k_ref = ktab.cpu().numpy()
    log = s.integrate_logged(conc, ktab, w.dt, log_cap=8192)
    torch.cuda.synchronize()
    ln = log["log_n"].cpu().numpy()
    ok = (log["status"].cpu().numpy() == 0) & (ln < 8192)
    rep = o.integrate(w.conc.copy(), w.dt, k=k_ref, dk=dk, temp=w.temp, rho=w.rho, rh=w.rh, param=w.param,
                      replay=(log["log_h"].cpu().numpy(), log["log_acc"].cpu().numpy(), ln))
    ok &= rep["status"] == 0
    assert ok.mean() > 0.9
    got, ref = conc.cpu().numpy()[:, ok], rep["conc"][:, ok]
    atol = np.array(o.raw["atol"])[:, None]
    assert (np.abs(got - ref) / (np.abs(ref) + atol)).max() <= 1e-9


def test_ts1_tendencies_and_jacobian(ts1_lib):
    """The table-driven evaluation entries (mkpp_evaluate_rates /
    mkpp_evaluate_jacobian: Mech::eval_step per cell, then the fixed-species
    columns) against the oracle: 1e-10 of the cell's largest entry, as for
    the unrolled mechanisms."""
    from mkpp_gb300.api import MechanismContext

    w = workloads.make("ts1", 4)
    o = Oracle("ts1")
    F_ref, J_ref = o.evaluate(w.conc, w.temp, w.rho, w.rh, None, w.param)
    Jd_ref = o.dense_jacobian(J_ref)          # [row, col, cell]
    ctx = MechanismContext("ts1", 4)
    try:
        ctx.set_state(np.ascontiguousarray(w.conc), w.temp.copy(), w.pressure.copy(), w.rho.copy())
        ctx.set_aerosol(relative_humidity=w.rh.copy())
        ctx.set_rate_parameters(np.ascontiguousarray(w.param))
        F = ctx.evaluate_rates()
        J = ctx.evaluate_jacobian()            # [col, row, cell]
    finally:
        ctx.close()
    assert np.all(np.abs(F - F_ref) <= 1e-10 * (np.abs(F_ref).max(axis=0) + 1e-300))
    Jt = np.transpose(J, (1, 0, 2))
    assert np.all(np.abs(Jt - Jd_ref) <= 1e-10 * (np.abs(Jd_ref).max(axis=(0, 1)) + 1e-300))

"""GPU runs at the benchmark configurations' full sizes.

The oracle cannot integrate 262144 SAPRC99 cells in a test's time, so the
full-size runs are checked through a size-independent property.  Subset
independence: every cell's result is bit-identical whether it is integrated
in the full batch or in a batch of a sample of cells spread over the whole
index range.  That catches indexing, work-queue, scratch-tile and parking
errors that appear only at scale.  Bit-identity holds by design: cells are
independent, and the lane, warp or kernel that runs a cell does not change
its arithmetic (the plain/persistent and cooperative hand-off tests check
that directly).

Chapman's full configuration (4096 cells) is small enough for the oracle,
with the step sequence forced, per species to 1e-9.
"""
import numpy as np
import pytest

from mkpp_gb300 import workloads

pytestmark = pytest.mark.gpu

# (mechanism, cells, host steps): small_strato's whole configuration; for
# SAPRC99 all cells over the first (stiffest) host step.
FULL = [("small_strato", 65536, 12), ("saprc99", 262144, 1)]
SAMPLE = 1024


def _window(w, host_steps):
    """One persistent launch over `host_steps` host steps, as bench.py runs it:
    the rate constants of every host step first, the first step's status
    passed on."""
    import torch

    from mkpp_gb300.api import DeviceSolver

    s = DeviceSolver(w.mechanism)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    n, nr = w.ncells, s.sizes.reactions
    conc = d(w.conc)
    ktab = torch.empty((host_steps, nr, n), dtype=torch.float64, device="cuda")
    status = None
    for h in range(host_steps):
        k, st = s.rate_constants(conc, d(w.temp), d(w.rho), d(w.rh), None, d(w.param_at(h)))
        ktab[h].copy_(k)
        if status is None:
            status = st
    acc = torch.zeros(n, dtype=torch.int32, device="cuda")
    rej = torch.zeros_like(acc)
    s.integrate_k(conc, ktab, w.dt, steps=host_steps, k_step_stride=nr * n, status=status, accepted=acc,
                  rejected=rej)
    torch.cuda.synchronize()
    return conc.cpu().numpy(), status.cpu().numpy(), (acc + rej).cpu().numpy()


def _sample(w, idx):
    """The workload restricted to cells `idx` (same seeded draws)."""
    pick = lambda a: np.ascontiguousarray(a[..., idx])  # noqa: E731
    return workloads.Workload(w.name, w.mechanism, pick(w.conc), pick(w.temp), pick(w.pressure), pick(w.rho),
                              pick(w.rh), pick(w.param), w.dt, w.host_steps,
                              None if w.phase is None else pick(w.phase), w.jmax, dict(w.extra))


@pytest.mark.parametrize("mech,cells,host_steps", FULL)
def test_full_batch_equals_sampled_batch(built_libs, mech, cells, host_steps):
    w = workloads.make(mech, cells)
    full_conc, full_status, full_att = _window(w, host_steps)
    rng = np.random.default_rng(11)
    idx = np.sort(rng.choice(cells, size=SAMPLE, replace=False))
    idx[-1] = cells - 1                      # the last cell, where index errors show
    sub_conc, sub_status, sub_att = _window(_sample(w, idx), host_steps)
    assert np.array_equal(full_conc[:, idx], sub_conc, equal_nan=True)
    assert np.array_equal(full_status[idx], sub_status)
    assert np.array_equal(full_att[idx], sub_att)


def test_chapman_full_configuration_forced_steps(built_libs):
    import torch

    from mkpp_gb300.api import DeviceSolver
    from oracle.oracle import Oracle

    w = workloads.make("chapman")             # 4096 cells, one 3600 s host step
    assert w.ncells == 4096
    s, o = DeviceSolver("chapman"), Oracle("chapman")
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    conc = d(w.conc)
    ktab, _ = s.rate_constants(conc, d(w.temp), d(w.rho), d(w.rh), None, d(w.param))
    log = s.integrate_logged(conc, ktab, w.dt, log_cap=8192)
    torch.cuda.synchronize()
    ln = log["log_n"].cpu().numpy()
    ok = (log["status"].cpu().numpy() == 0) & (ln < 8192)
    rep = o.integrate(w.conc.copy(), w.dt, temp=w.temp, rho=w.rho, rh=w.rh, param=w.param,
                      replay=(log["log_h"].cpu().numpy(), log["log_acc"].cpu().numpy(), ln))
    ok &= rep["status"] == 0
    assert ok.mean() > 0.9
    got, ref = conc.cpu().numpy()[:, ok], rep["conc"][:, ok]
    atol = np.array(o.raw["atol"])[:, None]
    assert (np.abs(got - ref) / (np.abs(ref) + atol)).max() <= 1e-9

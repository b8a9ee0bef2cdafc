"""Launch tuning on a live handle (mkpp_set_launch_tuning between calls)."""
import numpy as np
import pytest

from mkpp_gb300 import workloads

pytestmark = pytest.mark.gpu


def test_launch_tuning_change_on_a_live_handle(built_libs):
    """mkpp_integrate, then mkpp_set_launch_tuning to the 128-register variant
    (twice the resident blocks, so a larger integrate scratch for SAPRC99's
    global tile store), then mkpp_integrate again on the same handle and
    inputs: the handle's scratch grows and the results are identical."""
    from mkpp_gb300.api import DeviceSolver, MechanismContext

    w, s = workloads.make("saprc99", 48), DeviceSolver("saprc99")
    ctx = MechanismContext("saprc99", w.ncells)
    outs = []
    try:
        for rv in (2, 4):
            s.set_tuning(register_variant=rv)
            host = np.ascontiguousarray(w.conc.copy())
            ctx.set_state(host, w.temp.copy(), w.pressure.copy(), w.rho.copy())
            ctx.set_aerosol(relative_humidity=w.rh.copy())
            ctx.set_rate_parameters(np.ascontiguousarray(w.param))
            ctx.integrate(w.dt)
            outs.append(host.copy())
    finally:
        s.set_tuning(register_variant=2)
        ctx.close()
    assert np.array_equal(outs[0], outs[1], equal_nan=True)


def test_cost_order_leaves_results_unchanged(built_libs):
    """mkpp_set_cost_order: three host steps through mkpp_integrate with the
    previous call's most expensive cells handed out first end bit-identical,
    state and per-cell counts, to the same calls in cell order."""
    from mkpp_gb300.api import MechanismContext

    w = workloads.make("saprc99", 96)
    runs = []
    for enable in (False, True):
        ctx = MechanismContext("saprc99", w.ncells)
        try:
            ctx.set_cost_order(enable)
            host = np.ascontiguousarray(w.conc.copy())
            ctx.set_state(host, w.temp.copy(), w.pressure.copy(), w.rho.copy())
            ctx.set_aerosol(relative_humidity=w.rh.copy())
            out = []
            for step in range(3):
                ctx.set_rate_parameters(np.ascontiguousarray(w.param_at(step)))
                ctx.integrate(w.dt)
                out.append((host.copy(), *ctx.cell_stats()))
            runs.append(out)
        finally:
            ctx.close()
    for a, b in zip(*runs):
        for x, y in zip(a, b):
            assert np.array_equal(x, y, equal_nan=True)


@pytest.mark.parametrize("mech", ["small_strato", "saprc99"])
def test_tail_parking_leaves_results_unchanged(built_libs, mech):
    """mkpp_set_tail_parking: with 96 cells every cell is handed out at once
    and fewer cells are on lanes than the cooperative kernel runs, so every
    cell past 32 attempts is parked at its next multiple of 16 attempts.
    State, status and attempt counts end bit-identical to the run without
    tail parking (a window of 2 host steps)."""
    import torch

    from mkpp_gb300.api import DeviceSolver

    w, s = workloads.make(mech, 96), DeviceSolver(mech)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    outs = []
    try:
        for tail in (0, 32):
            s.set_tail_parking(tail)
            conc = d(w.conc)
            st, acc, rej = s.integrate(conc, w.dt, steps=2, temp=d(w.temp), rho=d(w.rho), rh=d(w.rh),
                                       param=d(w.param), mode="persistent")
            torch.cuda.synchronize()
            outs.append((conc.cpu().numpy(), st.cpu().numpy(), acc.cpu().numpy(), rej.cpu().numpy()))
    finally:
        s.set_tail_parking(0)
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("mech", ["small_strato", "saprc99"])
def test_split_launch_leaves_results_unchanged(built_libs, mech):
    """mkpp_set_split_launch: the first cells of the order on whole warps of
    reserved SMs, the rest on the persistent body (a window of 2 host steps,
    640 cells, the order reversed, its first 40 cells on 4 SMs).  State,
    status, attempt counts and carried step sizes end bit-identical to the
    launch without the split, with and without step-size carry-over."""
    import torch

    from mkpp_gb300.api import DeviceSolver

    n = 640
    w, s = workloads.make(mech, n), DeviceSolver(mech)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    conc0 = d(w.conc)
    nr = s.sizes.reactions
    ktab = torch.empty((2, nr, n), dtype=torch.float64, device="cuda")
    for h in range(2):
        k, _ = s.rate_constants(conc0, d(w.temp), d(w.rho), d(w.rh), None, d(w.param_at(h)))
        ktab[h].copy_(k)
    order = torch.arange(n - 1, -1, -1, dtype=torch.int32, device="cuda")
    for carry in (False, True):
        outs = []
        try:
            for split in ((0, 0), (40, 4)):
                s.set_split_launch(*split)
                conc = conc0.clone()
                st = torch.zeros(n, dtype=torch.int32, device="cuda")
                acc, rej = torch.zeros_like(st), torch.zeros_like(st)
                dtc = torch.zeros(n, dtype=torch.float64, device="cuda") if carry else None
                s.integrate_k(conc, ktab, w.dt, steps=2, k_step_stride=nr * n, status=st, accepted=acc,
                              rejected=rej, order=order, dt_carry=dtc)
                torch.cuda.synchronize()
                outs.append([x.cpu().numpy() for x in (conc, st, acc, rej) + ((dtc,) if carry else ())])
        finally:
            s.set_split_launch(0, 0)
        for a, b in zip(outs[0], outs[1]):
            assert np.array_equal(a, b, equal_nan=True)

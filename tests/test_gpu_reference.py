"""GPU results against the reference's own generated solver, same inputs.

The GPU kernels are compared with the CPU oracle elsewhere (forced step
sequences to 1e-9), and the oracle with the reference's generated
integrate() (tests/test_oracle_reference.py).  Here the two ends meet
directly: the reference's SolverKernels<D>::integrate(), regenerated by its
compiler and built on the host cores (oracle/ref_build.py, the same build
bench.py times as the CPU baseline), against the GPU's free-running
integrate on the same seeded cells, with the ROS-3 tableau and, for Chapman
and small_strato, RODAS-3 (the reference compiler's --solver rodas3 against
the *_rodas3 libraries).  Skipped where that build is absent.

Free-running, an accept/reject decision can flip on round-off, after which a
cell follows another step sequence within the tolerances, so the bounds are
those of the free-running oracle test: every species within
10 (rtol |ref| + atol), and the median relative difference at round-off.
SAPRC99 keeps its shipped 1e33-1e37 1/s rates here (the reference evaluates
them itself), so it gets statistical bounds: >= 90% of cells finite on both
sides, median <= 1e-9, worst cell <= 1e-2 relative.
"""
import numpy as np
import pytest

from mkpp_gb300 import workloads

pytestmark = pytest.mark.gpu

CELLS = {"chapman": 512, "small_strato": 512, "saprc99": 48, "chapman_rodas3": 512, "small_strato_rodas3": 512,
         "ts1": 32}


def _run(mech):
    import torch

    from mkpp_gb300.api import DeviceSolver
    from mkpp_gb300.emitter.plan import load_raw
    from oracle import ref_build

    ref = ref_build.load(mech) if mech in ref_build.MECHS else ref_build.ensure(mech)
    if ref is None:
        pytest.skip("the reference's generated solver is not built on this machine")
    w = workloads.make(mech, CELLS[mech])
    s = DeviceSolver(mech)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    conc = d(w.conc)
    st, _, _ = s.integrate(conc, w.dt, temp=d(w.temp), rho=d(w.rho), rh=d(w.rh), param=d(w.param))
    torch.cuda.synchronize()
    rr = ref.integrate(w.conc.copy(), w.dt, 1, temp=w.temp, rho=w.rho, rh=w.rh, param=w.param)
    raw = load_raw(mech)
    got, ref_conc = conc.cpu().numpy(), rr["conc"]
    ok = (st.cpu().numpy() == 0) & np.isfinite(ref_conc).all(axis=0) & np.isfinite(got).all(axis=0)
    return got, ref_conc, ok, np.array(raw["rtol"])[:, None], np.array(raw["atol"])[:, None]


@pytest.mark.parametrize("mech", ["chapman", "small_strato", "chapman_rodas3", "small_strato_rodas3"])
def test_free_running_matches_reference_solver(built_libs, mech):
    got, ref, ok, rtol, atol = _run(mech)
    assert ok.mean() > 0.9
    g, r = got[:, ok], ref[:, ok]
    assert np.all(np.abs(g - r) <= 10 * (rtol * np.abs(r) + atol))
    assert np.median(np.abs(g - r) / (np.abs(r) + atol)) <= 1e-9


def test_free_running_matches_reference_solver_saprc99(built_libs):
    got, ref, ok, rtol, atol = _run("saprc99")
    assert ok.mean() >= 0.9
    rel = np.abs(got - ref)[:, ok] / np.maximum(np.abs(ref[:, ok]), 1.0)
    assert np.median(rel) <= 1e-9
    assert rel.max() <= 1e-2


def test_free_running_matches_reference_solver_ts1():
    """TS1 (table-driven library) against the reference's own TS1 solver at
    the plan's tolerances, 32 cells over one 600 s host step, with the
    shipped 1e29-1e41 1/s rates: every cell finite on both sides, every
    species within 10 (rtol |ref| + atol), the median relative difference
    (|ref| + atol) at most 1e-9."""
    from mkpp_gb300 import build

    build.build(("ts1",))
    got, ref, ok, rtol, atol = _run("ts1")
    assert ok.all()
    d = np.abs(got - ref)
    assert np.all(d <= 10 * (rtol * np.abs(ref) + atol))
    assert np.median(d / (np.abs(ref) + atol)) <= 1e-9

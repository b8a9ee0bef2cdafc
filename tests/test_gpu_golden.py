"""The GPU against the reference's own golden outputs for this path, with no
oracle in between (the oracle meets the same vectors in
tests/test_oracle_golden.py):
* the reference's native Chapman run
  (reports/native-kokkos-5.1.1/final-mkpp-chapman.stdout.json, fixture
  tests/golden/chapman_kokkos_10x60.json): one cell, 10 x integrate(60 s) at
  the shipped tolerances (rtol 1e-6, atol 1e-3), through the chapman_shipped
  library (the Chapman plan exported at those tolerances).  The oracle
  matches it to 1e-14; the GPU is held to 1e-9;
* the SciPy-Radau Chapman solution of the reference's e2e test
  (tests/integration/e2e_validation/data/chapman_reference.json, fixture
  tests/golden/chapman_scipy_reference.json) under the reference's own gate
  |d| <= 1 + 1e-4 |ref| (test_scipy_validation.cpp:246-247), through the
  chapman library (rtol 1e-3, atol 1).
"""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def libs():
    from mkpp_gb300 import build

    return build.build(("chapman", "chapman_shipped"))


def _solve(mech, conc0, jvals, dt, steps):
    import torch

    from mkpp_gb300.api import DeviceSolver

    s = DeviceSolver(mech)
    conc = torch.tensor(np.asarray(conc0, dtype=np.float64)[:, None], device="cuda").contiguous()
    param = torch.tensor(np.asarray(jvals, dtype=np.float64)[:, None], device="cuda").contiguous()
    st, _, _ = s.integrate(conc, dt, steps=steps, param=param)
    torch.cuda.synchronize()
    return conc.cpu().numpy()[:, 0], int(st.cpu().numpy()[0])


def test_reference_native_chapman_run(libs):
    from mkpp_gb300.emitter.plan import load_raw

    g = json.loads((GOLD / "chapman_kokkos_10x60.json").read_text())
    names = load_raw("chapman_shipped")["species"]
    got, status = _solve("chapman_shipped", [g["initial"][s] for s in names], g["jvals"], g["dt"], g["steps"])
    want = np.array([g["final"][s] for s in names])
    assert status == 0
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=0)


def test_reference_scipy_radau_gate(libs):
    g = json.loads((GOLD / "chapman_scipy_reference.json").read_text())
    got, status = _solve("chapman", g["initial_conditions"], g["jvals"], g["time_span"][1], 1)
    want = np.array(g["expected_final"])
    assert status == 0
    assert np.all(np.abs(got - want) <= g["gate"]["atol"] + g["gate"]["rtol"] * np.abs(want))

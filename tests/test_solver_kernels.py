"""The generated C++ solver API: SolverKernels<DeviceType> per mechanism.

generated/host_api/<m>/<m>.hpp + include/mkpp_gb300/solver_kernels.hpp keep
the reference's generated SolverKernels members (src/mkpp/templates/header.j2:
127-203, solver_variants/integrate.j2:52-67, kernel_functions/compute_*.j2)
and route them to the mechanism library.  tests/solver_kernels/
solver_kernels_check.cpp calls them from a dispatcher-shaped call site
(src/mkpp_host/include/mkpp_host/dispatcher.hpp:101-122,225-254), compiled
with g++ -std=c++20 as the reference's host code is.

* CPU: the call site compiles against every mechanism's header (both device
  types, the environment forms each mechanism's constants select, the
  MKPP_ENABLE_ADJOINT members); the constants equal the plan's; without a
  GPU the first solve fails loudly (no CPU fallback).
* GPU: per cell, integrate() through the deferred and the synchronous device
  types, the host registry's execute() and the C ABI driven from Python end
  bit for bit alike; compute_rates / compute_jacobian / compute_tlm /
  compute_adjoint equal the C ABI's evaluation entries bit for bit, and the
  Jacobian is written exactly at the reference's sparse pattern.
"""
import os
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from mkpp_gb300 import workloads
from mkpp_gb300.emitter.plan import load_raw

ROOT = Path(__file__).resolve().parent.parent
GEN = ROOT / "mkpp_gb300" / "generated" / "host_api"
LIB = ROOT / "mkpp_gb300" / "lib"
MECHS = ("chapman", "small_strato", "saprc99", "ts1", "saprc99_mini", "saprcnov", "chapman_shipped")


def _compile(mech: str, out: Path) -> Path:
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    raw = load_raw(mech)
    exe = out / f"solver_kernels_{mech}"
    cmd = ["g++", "-std=c++20", "-O1", "-fopenmp", "-Wall", "-Wextra", "-Werror", "-DMKPP_ENABLE_ADJOINT",
           f"-I{ROOT / 'include'}", f"-I{ROOT / 'oracle' / 'kokkos_shim'}", f"-I{GEN / mech}",
           f'-DMKPP_KERNELS_HEADER="{mech}.hpp"', f"-DMKPP_KERNELS_NS=mkpp::generated::{mech}",
           f"-DMKPP_NUM_SPECIES_CHECK={len(raw['species'])}",
           str(ROOT / "tests" / "solver_kernels" / "solver_kernels_check.cpp"), "-ldl", "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("mech", MECHS)
def test_call_site_compiles_and_constants_match_plan(mech, tmp_path):
    _compile(mech, tmp_path)
    raw = load_raw(mech)
    text = (GEN / mech / f"{mech}.hpp").read_text()
    species = re.findall(r"^    (\w+) = (\d+)", text, re.M)
    assert [s for s, _ in species] == raw["species"]
    assert [int(i) for _, i in species] == list(range(len(raw["species"])))
    const = dict(re.findall(r"static constexpr \w+ (\w+) = ([^;\[]+);", text))
    assert int(const["NUM_RUNTIME_PARAMETERS"]) == raw["num_rate_parameters"]
    assert int(const["NUM_PHOTOLYSIS"]) == raw["num_photolysis"]
    assert const["SUPPORTS_RUNTIME_ENVIRONMENT"] == ("true" if raw["runtime_environment"] else "false")
    assert const["HAS_CLOUD_GATED"] == ("true" if raw["cloud_gated"] else "false")
    assert float(const["INITIAL_STEP_SEED"]) == raw["initial_step_seed"]
    atol = [float(x) for x in re.search(r"atol\[NUM_SPECIES\] = \{([^}]*)\}", text).group(1).split(",")]
    rtol = [float(x) for x in re.search(r"rtol\[NUM_SPECIES\] = \{([^}]*)\}", text).group(1).split(",")]
    assert atol == raw["atol"] and rtol == raw["rtol"]


def _cuda():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def _inputs(mech: str, n: int, d: Path):
    w = workloads.make(mech, n)
    for name, a in (("conc", w.conc), ("temp", w.temp), ("rh", w.rh), ("rho", w.rho), ("param", w.param)):
        np.ascontiguousarray(a, dtype=np.float64).tofile(d / f"{name}.bin")
    return w


def test_without_gpu_the_first_solve_fails_loudly(tmp_path):
    if _cuda():
        pytest.skip("a GPU is present")
    from mkpp_gb300 import build

    try:
        build.build(("chapman",))
    except RuntimeError as e:  # no nvcc
        pytest.skip(str(e))
    exe = _compile("chapman", tmp_path)
    _inputs("chapman", 4, tmp_path)
    out = subprocess.run([str(exe), str(tmp_path), "4", "60", "1"], capture_output=True, text=True,
                         env={**os.environ, "MKPP_GB300_LIB_DIR": str(LIB)})
    assert out.returncode == 3, out.stderr
    assert "FATAL ERROR" in out.stderr


# TS1 runs 4 cells over 60 s: its synchronous form solves one cell per
# call, each on a single lane of the table-driven attempt.
@pytest.mark.gpu
@pytest.mark.parametrize("mech,n,steps,dt", [("chapman", 256, 2, None), ("small_strato", 256, 2, None),
                                             ("saprc99", 64, 1, None), ("ts1", 4, 1, 60.0)])
def test_solver_kernels_match_c_abi(mech, n, steps, dt, tmp_path):
    from mkpp_gb300 import build
    from mkpp_gb300.api import MechanismContext

    build.build((mech,))
    exe = _compile(mech, tmp_path)
    w = _inputs(mech, n, tmp_path)
    if dt is not None:
        w.dt = dt
    out = subprocess.run([str(exe), str(tmp_path), str(n), repr(w.dt), str(steps)], capture_output=True, text=True,
                         env={**os.environ, "MKPP_GB300_LIB_DIR": str(LIB)})
    assert out.returncode == 0, out.stderr
    ns = w.conc.shape[0]
    rd = lambda name, shape: np.fromfile(tmp_path / f"{name}.bin").reshape(shape)  # noqa: E731

    # The C ABI on the same inputs, driven from Python.
    host = np.ascontiguousarray(w.conc.copy())
    ctx = MechanismContext(mech, n)
    try:
        ctx.set_state(host, w.temp.copy(), w.pressure.copy(), w.rho.copy())
        ctx.set_aerosol(relative_humidity=w.rh.copy())
        ctx.set_rate_parameters(np.ascontiguousarray(w.param))
        st = np.zeros(n, np.int32)
        for s in range(steps):
            ctx.integrate(w.dt)
            st_s, _, _ = ctx.cell_stats()
            st = np.where(st == 0, st_s, st)
        evals = MechanismContext(mech, n)
        try:
            c0 = np.ascontiguousarray(w.conc.copy())
            evals.set_state(c0, w.temp.copy(), w.pressure.copy(), w.rho.copy())
            evals.set_aerosol(relative_humidity=w.rh.copy())
            evals.set_rate_parameters(np.ascontiguousarray(w.param))
            F = evals.evaluate_rates()
            J = evals.evaluate_jacobian()              # [col, row, cell]
            JV = evals.evaluate_jacobian_vector(c0)
        finally:
            evals.close()
    finally:
        ctx.close()

    nan = lambda a: np.nan_to_num(a, nan=1.25e300)  # noqa: E731
    for name in ("deferred", "sync", "registry"):
        got = rd(name, (ns, n))
        assert np.array_equal(nan(got), nan(host)), name
    assert np.array_equal(rd("status", (n,)).astype(np.int32), st)
    assert np.array_equal(rd("rates", (ns, n)), F)
    assert np.array_equal(rd("tlm", (ns, n)), JV)
    jac = rd("jacobian", (ns, ns, n))              # [col, row, cell], as J
    adj = rd("adjoint", (ns, ns, n))               # J_adj(i, j) = J(j, i) at [j, i, cell]
    mask = np.zeros((ns, ns), bool)
    for i, j in load_raw(mech)["jacobian_entries"]:
        mask[j, i] = True
    assert np.array_equal(jac[mask], J[mask])
    assert not np.any(jac[~mask]) and not np.any(J[~mask])
    assert np.array_equal(adj, np.transpose(jac, (1, 0, 2)))

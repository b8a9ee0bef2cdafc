"""The C++ host registry (include/mkpp_host/mechanism_manager.hpp).

It mirrors the reference's MechanismRegistry and HostExecutionParams
(src/mkpp_host/include/mkpp_host/mechanism_manager.hpp:21-228,
dispatcher.hpp:15-254) over the mechanism libraries.  Checked through
tests/registry/registry_check.cpp:
* on the CPU: the registered mechanisms are the libraries built; get_info
  reports the library's sizes; an unknown name, a per-cell extent that does
  not match the state and too few forcing slots raise the reference's
  "FATAL ERROR" messages as std::runtime_error / std::invalid_argument;
* on the GPU: execute() with per-cell meteorology and forcing ends
  bit-identical to the C ABI driven from Python on the same inputs, and the
  batched path (execute_mechanism_steps_batched) leaves a cell with a NaN
  input untouched, flags it ERR_NON_FINITE_STATE (2), prints one summary
  line and integrates the others as the C ABI does
  (test_e2e_batched.cpp's NaN isolation).
"""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
LIB = ROOT / "mkpp_gb300" / "lib"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from mkpp_gb300 import build

    try:
        build.build(("chapman", "small_strato"))
    except RuntimeError as e:  # no nvcc
        pytest.skip(str(e))
    exe = tmp_path_factory.mktemp("registry") / "registry_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "registry" / "registry_check.cpp"), "-ldl", "-o", str(exe)], check=True)
    return exe


def _run(exe, *args):
    return subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True,
                          env={**os.environ, "MKPP_GB300_LIB_DIR": str(LIB)})


def test_registered_mechanisms_are_the_built_libraries(checker):
    out = _run(checker, "list")
    assert out.returncode == 0, out.stderr
    built = sorted(p.name[len("libmkpp_"):-len(".so")] for p in LIB.glob("libmkpp_*.so"))
    assert out.stdout.split() == built
    assert {"chapman", "small_strato"} <= set(built)


def test_get_info_reports_library_sizes(checker):
    from mkpp_gb300.emitter.plan import load_raw

    for mech in ("chapman", "small_strato"):
        out = _run(checker, "info", mech)
        assert out.returncode == 0, out.stderr
        raw = load_raw(mech)
        assert out.stdout.split() == [mech, str(len(raw["species"])), str(raw["num_reactions"]), "0"]


def test_unknown_mechanism_is_a_fatal_runtime_error(checker):
    out = _run(checker, "unknown", "no_such_mechanism")
    assert out.returncode == 3
    assert out.stdout.startswith("FATAL ERROR: Unknown mechanism 'no_such_mechanism'. Supported: ")
    assert "chapman" in out.stdout


def test_extent_checks_raise_invalid_argument(checker):
    out = _run(checker, "extent", "chapman")
    assert out.returncode == 3
    assert out.stdout.strip() == "FATAL ERROR: per-cell meteorology extent does not match state"
    out = _run(checker, "forcing", "chapman")
    assert out.returncode == 3
    assert out.stdout.strip() == "FATAL ERROR: per-cell forcing has too few runtime parameters"


@pytest.mark.gpu
@pytest.mark.parametrize("mech", ["chapman", "small_strato"])
def test_execute_matches_c_abi(checker, mech, tmp_path):
    from mkpp_gb300 import workloads
    from mkpp_gb300.api import MechanismContext

    n, steps = 256, 2
    w = workloads.make(mech, n)
    for name, a in (("conc", w.conc), ("temp", w.temp), ("rho", w.rho), ("rh", w.rh), ("param", w.param)):
        np.ascontiguousarray(a, dtype=np.float64).tofile(tmp_path / f"{name}.bin")
    out = _run(checker, "execute", mech, n, repr(w.dt), steps, tmp_path)
    assert out.returncode == 0, out.stderr
    got = np.fromfile(tmp_path / "conc_out.bin").reshape(w.conc.shape)
    status = np.fromfile(tmp_path / "status.bin", dtype=np.int32)
    ref = np.ascontiguousarray(w.conc.copy())
    ctx = MechanismContext(mech, n)
    first = np.zeros(n, np.int32)
    try:
        ctx.set_state(ref, w.temp.copy(), np.full(n, 101325.0), w.rho.copy())
        ctx.set_aerosol(relative_humidity=w.rh.copy())
        ctx.set_rate_parameters(np.ascontiguousarray(w.param))
        for _ in range(steps):
            ctx.integrate(w.dt)
            st = ctx.cell_stats()[0]
            first = np.where(first == 0, st, first)
    finally:
        ctx.close()
    assert np.array_equal(got, ref, equal_nan=True)
    # execute() reports each cell's first failure over the steps.
    assert np.array_equal(status, first)


@pytest.mark.gpu
def test_batched_path_isolates_non_finite_cell(checker, tmp_path):
    from mkpp_gb300 import workloads
    from mkpp_gb300.api import MechanismContext

    mech, n, steps, bad = "chapman", 64, 1, 5
    w = workloads.make(mech, n)
    conc = np.ascontiguousarray(w.conc.copy())
    conc[0, bad] = np.nan
    jvals = np.ascontiguousarray(w.param[:, 0])
    conc.tofile(tmp_path / "conc.bin")
    jvals.tofile(tmp_path / "jvals.bin")
    out = _run(checker, "batched", mech, n, repr(w.dt), steps, tmp_path)
    assert out.returncode == 0, out.stderr
    assert f"reported 1 faulted cell(s) of {n}" in out.stderr
    got = np.fromfile(tmp_path / "conc_out.bin").reshape(conc.shape)
    status = np.fromfile(tmp_path / "status.bin", dtype=np.int32)
    assert status[bad] == 2 and (np.delete(status, bad) == 0).all()
    assert np.array_equal(got[:, bad], conc[:, bad], equal_nan=True)
    ref = conc.copy()
    ctx = MechanismContext(mech, n)
    try:
        ctx.set_state(ref, np.full(n, 288.15), np.full(n, 101325.0), np.full(n, 2.4476e19))
        ctx.set_aerosol(relative_humidity=np.full(n, 0.5))
        ctx.set_rate_parameters(np.ascontiguousarray(np.repeat(jvals[:, None], n, axis=1)))
        ctx.integrate(w.dt)
    finally:
        ctx.close()
    assert np.array_equal(got, ref, equal_nan=True)


def test_registry_builds_with_nvtx_ranges(tmp_path):
    """With the CUDA toolkit's include directory on the path, the header opens
    the reference's NVTX range MKPP_Batched_Team_Dispatch_<name>
    (dispatcher.hpp:335) around the batched dispatch; it still builds without
    warnings and finds the libraries."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from mkpp_gb300 import build

    try:
        cuda_inc = Path(build.nvcc()).resolve().parent.parent / "include"
        build.build(("chapman",))
    except RuntimeError as e:  # no nvcc
        pytest.skip(str(e))
    if not (cuda_inc / "nvtx3" / "nvToolsExt.h").exists():
        pytest.skip("no NVTX3 headers in the CUDA toolkit")
    header = (ROOT / "include" / "mkpp_host" / "mechanism_manager.hpp").read_text()
    assert 'TraceRange range("MKPP_Batched_Team_Dispatch_" + name)' in header
    exe = tmp_path / "registry_check_nvtx"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
                    f"-I{cuda_inc}", str(ROOT / "tests" / "registry" / "registry_check.cpp"), "-ldl", "-o", str(exe)],
                   check=True)
    out = _run(exe, "list")
    assert out.returncode == 0 and "chapman" in out.stdout.split(), out.stderr

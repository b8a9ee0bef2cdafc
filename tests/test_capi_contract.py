"""C-ABI lifecycle and argument contract, on any host (no GPU needed).

The reference's contract tests (tests/contract/test_c_abi.cpp:9-80) check the
handle lifecycle, state binding and error codes of the generated mkpp.h.
The same calls against libmkpp_chapman.so, plus the argument checks that
return before any device work (src/mkpp/templates/host_api/
mkpp_c_api.cpp.j2:70-374 gives the codes):
* null handles and pointers: MKPP_ERROR_NULL_POINTER (-101);
* zero cells, a wrong parameter count, dt <= 0, a non-positive temperature:
  MKPP_ERROR_INVALID_ARGUMENT (-103), with a "FATAL ERROR" message;
* integrate or evaluate before initialization, statistics before any
  integration: MKPP_ERROR_INVALID_STATE (-104);
* an unknown species name: MKPP_ERROR_NOT_FOUND (-106).
Initialization makes no CUDA call, as the reference's makes no device call.
The first call that computes does: on a host without a GPU it fails loudly
with MKPP_ERROR_DEVICE (-107) and the CUDA runtime's reason (there is no CPU
fallback); on a GB300 it succeeds.
"""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent

MECH = "chapman"


@pytest.fixture(scope="module")
def lib():
    from mkpp_gb300 import api, build

    try:
        build.build((MECH,))
    except RuntimeError as e:  # no nvcc
        pytest.skip(str(e))
    return api.load_library(MECH)


def _handle(lib, n):
    h = C.c_void_p()
    assert lib.mkpp_create_handle(C.byref(h), n) == 0
    assert h.value
    return h


def _error(lib, h):
    buf = C.create_string_buffer(512)
    assert lib.mkpp_get_last_error(h, buf, 512) == 0
    return buf.value.decode()


def _gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:  # noqa: BLE001
        return False


def test_handle_lifecycle_and_metadata(lib):
    assert lib.mkpp_initialize(None) == -101
    h = C.c_void_p()
    assert lib.mkpp_create_handle(None, 10) == -101
    assert lib.mkpp_create_handle(C.byref(h), 0) == -103
    h = _handle(lib, 10)
    assert lib.mkpp_initialize(h) == 0
    count = C.c_size_t()
    assert lib.mkpp_get_species_count(h, C.byref(count)) == 0 and count.value == 4
    assert lib.mkpp_get_reaction_count(h, C.byref(count)) == 0 and count.value == 4
    assert lib.mkpp_get_photolysis_count(h, C.byref(count)) == 0 and count.value == 2
    assert lib.mkpp_get_species_count(h, None) == -101
    idx = C.c_int(-1)
    assert lib.mkpp_get_species_index(h, b"O3", C.byref(idx)) == 0 and idx.value == 2
    assert lib.mkpp_get_species_index(h, b"XYZ", C.byref(idx)) == -106
    assert lib.mkpp_destroy_handle(h) == 0
    assert lib.mkpp_destroy_handle(None) == -101


def test_state_binding_and_argument_errors(lib):
    n = 5
    h = _handle(lib, n)
    try:
        conc = np.full((4, n), 1e9)
        t, p, rho = np.full(n, 298.15), np.full(n, 101325.0), np.full(n, 2.45e19)
        ptr = lambda a: a.ctypes.data  # noqa: E731
        # Before initialization.
        assert lib.mkpp_set_state_ptrs(h, ptr(conc), ptr(t), ptr(p), ptr(rho)) == 0
        assert lib.mkpp_integrate(h, C.c_double(60.0)) == -104
        assert "initialized" in _error(lib, h)
        assert lib.mkpp_initialize(h) == 0
        assert lib.mkpp_set_state_ptrs(h, None, ptr(t), ptr(p), ptr(rho)) == -101
        assert lib.mkpp_set_state_ptrs(h, ptr(conc), ptr(t), ptr(p), ptr(rho)) == 0
        prm = np.zeros((2, n))
        assert lib.mkpp_set_rate_parameter_ptrs(h, ptr(prm), 3) == -103
        assert lib.mkpp_set_rate_parameter_ptrs(h, ptr(prm), 2) == 0
        rh, sa = np.full(n, 0.7), np.full(n, 1e-4)
        assert lib.mkpp_set_aerosol_ptrs(h, ptr(rh), ptr(sa)) == 0
        assert lib.mkpp_set_cloud_water_ptr(h, ptr(np.zeros(n))) == 0
        status = np.zeros(n, np.int32)
        assert lib.mkpp_get_cell_stats(h, ptr(status), None, None) == -104
        assert lib.mkpp_set_initial_step_seed(None, C.c_double(1e-6)) == -101
        for bad in (0.0, -1e-6, float("nan"), float("inf")):
            assert lib.mkpp_set_initial_step_seed(h, C.c_double(bad)) == -103
        assert "initial_step_seed" in _error(lib, h)
        assert lib.mkpp_set_initial_step_seed(h, C.c_double(1e-5)) == 0
        assert lib.mkpp_set_max_attempts(h, 0) == -103 and lib.mkpp_set_max_attempts(h, 5000) == 0
        assert lib.mkpp_set_cost_order(None, 1) == -101
        assert lib.mkpp_set_cost_order(h, 1) == 0 and lib.mkpp_set_cost_order(h, 0) == 0
        assert lib.mkpp_integrate(h, C.c_double(0.0)) == -103
        assert lib.mkpp_integrate(h, C.c_double(float("nan"))) == -103
        t[2] = 0.0
        assert lib.mkpp_integrate(h, C.c_double(60.0)) == -103
        assert _error(lib, h).startswith("FATAL ERROR: cell temperature")
        t[2] = 298.15
        assert lib.mkpp_evaluate_rates(h, None) == -101
        assert lib.mkpp_evaluate_jacobian(h, None) == -101
        v = np.zeros((4, n))
        assert lib.mkpp_evaluate_jacobian_vector(h, None, ptr(v)) == -101
        assert lib.mkpp_evaluate_jacobian_transpose_vector(h, ptr(v), None) == -101
        assert lib.mkpp_evaluate_jacobian_vector(None, ptr(v), ptr(v)) == -101
    finally:
        assert lib.mkpp_destroy_handle(h) == 0


def test_compute_without_a_gpu_fails_loudly(lib):
    n = 4
    h = _handle(lib, n)
    try:
        conc = np.full((4, n), 1e9)
        t, p, rho = np.full(n, 298.15), np.full(n, 101325.0), np.full(n, 2.45e19)
        prm = np.zeros((2, n))
        assert lib.mkpp_initialize(h) == 0
        assert lib.mkpp_set_state_ptrs(h, conc.ctypes.data, t.ctypes.data, p.ctypes.data, rho.ctypes.data) == 0
        assert lib.mkpp_set_rate_parameter_ptrs(h, prm.ctypes.data, 2) == 0
        rc = lib.mkpp_integrate(h, C.c_double(60.0))
        if _gpu():
            assert rc == 0
        else:
            assert rc == -107
            assert _error(lib, h).startswith("FATAL ERROR: cudaStreamCreateWithFlags")
            assert np.all(conc == 1e9)
    finally:
        assert lib.mkpp_destroy_handle(h) == 0


@pytest.mark.parametrize("mech", ["chapman", "ts1"])
def test_reference_contract_program_against_generated_header(mech, tmp_path):
    """tests/capi/c_abi_contract.c, the reference's test_c_abi.cpp cases
    written in C11, compiled with gcc against the mechanism's generated
    mkpp.h (mkpp_gb300/generated/host_api/<m>/, which adds MKPP_NUM_SPECIES
    and the other sizes to include/mkpp.h) and linked to its library."""
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    from mkpp_gb300 import build

    try:
        lib = build.build((mech,))[0]
    except RuntimeError as e:  # no nvcc
        pytest.skip(str(e))
    exe = tmp_path / "c_abi_contract"
    inc = ROOT / "mkpp_gb300" / "generated" / "host_api" / mech
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", f"-I{inc}",
                    str(ROOT / "tests" / "capi" / "c_abi_contract.c"), str(lib),
                    f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stderr


@pytest.mark.parametrize("mech", ["chapman", "ts1"])
def test_reference_cpp_wrapper_and_sizes(mech, tmp_path):
    """The reference's own generated host API for the mechanism (generated
    here by its compiler, oracle/ref_build.py; skipped where the reference
    is absent): its mkpp.h defines the same MKPP_NUM_* sizes as this
    repository's generated host_api/<m>/mkpp.h, and its C++ wrapper mkpp.hpp,
    unchanged, compiles against this repository's header and drives the
    library (tests/capi/cpp_wrapper_check.cpp)."""
    import re

    from oracle import ref_build

    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    try:
        gen = ref_build.generate(mech, host_api=True)
    except Exception as e:  # noqa: BLE001
        pytest.skip(f"reference host API not generated: {e}")
    if not (gen / "mkpp.hpp").exists():
        pytest.skip("reference host API not generated")
    from mkpp_gb300 import build

    lib = build.build((mech,))[0]
    ours = ROOT / "mkpp_gb300" / "generated" / "host_api" / mech
    sizes = lambda t: dict(re.findall(r"#define (MKPP_NUM_\w+)\s+(\d+)", t))  # noqa: E731
    assert sizes((ours / "mkpp.h").read_text()) == sizes((gen / "mkpp.h").read_text())
    (tmp_path / "mkpp.hpp").write_text((gen / "mkpp.hpp").read_text())
    exe = tmp_path / "cpp_wrapper_check"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", f"-I{ours}", f"-I{tmp_path}",
                    str(ROOT / "tests" / "capi" / "cpp_wrapper_check.cpp"), str(lib),
                    f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", (out.returncode, out.stderr)


@pytest.mark.parametrize("mech", ["chapman", "ts1"])
def test_mechanism_flags_and_tolerances(mech):
    """mkpp_mechanism_flags / mkpp_mechanism_tolerances give the reference's
    SolverKernels constants (SUPPORTS_RUNTIME_ENVIRONMENT, HAS_CLOUD_GATED,
    atol[] and rtol[] in physical species order) from the plan."""
    from mkpp_gb300 import api, build
    from mkpp_gb300.emitter.plan import load_raw

    try:
        build.build((mech,))
    except RuntimeError as e:  # no nvcc
        pytest.skip(str(e))
    lib = api.load_library(mech)
    raw = load_raw(mech)
    env, cloud = C.c_int(-1), C.c_int(-1)
    assert lib.mkpp_mechanism_flags(C.byref(env), C.byref(cloud)) == 0
    assert (env.value, cloud.value) == (int(raw["runtime_environment"]), int(raw["cloud_gated"]))
    assert lib.mkpp_mechanism_flags(None, None) == -101
    ns = len(raw["species"])
    atol, rtol = np.zeros(ns), np.zeros(ns)
    assert lib.mkpp_mechanism_tolerances(atol.ctypes.data, rtol.ctypes.data) == 0
    assert atol.tolist() == raw["atol"] and rtol.tolist() == raw["rtol"]


def test_device_entry_argument_checks(lib):
    """The device-pointer entries reject bad arguments before touching the
    device: null pointers -101; zero cells, more than INT32_MAX cells, and
    non-positive dt, steps, seed or attempt cap -103; a parameter count other
    than the mechanism's -103.  No pointer here is dereferenced."""
    buf = np.zeros(64)
    p = buf.ctypes.data
    big = 2 ** 31
    integ = lambda n, conc=p, steps=1, dt=60.0, seed=1e-6, cap=100: lib.mkpp_gpu_integrate_k(  # noqa: E731
        n, conc, p, 0, steps, dt, seed, cap, 1, None, None, None, None, p, 1 << 30, None)
    assert integ(4, conc=None) == -101
    assert integ(0) == -103 and integ(big) == -103
    assert integ(4, steps=0) == -103 and integ(4, dt=0.0) == -103 and integ(4, dt=float("nan")) == -103
    assert integ(4, seed=0.0) == -103 and integ(4, cap=0) == -103
    assert lib.mkpp_gpu_rate_constants(4, None, p, p, None, None, p, 2, p, None, None) == -101
    assert lib.mkpp_gpu_rate_constants(0, p, p, p, None, None, p, 2, p, None, None) == -103
    assert lib.mkpp_gpu_rate_constants(4, p, p, p, None, None, p, 3, p, None, None) == -103
    assert lib.mkpp_gpu_tangent(4, p, 8, None, p, p, p, None, p, p, 1 << 30, None) == -101
    assert lib.mkpp_gpu_tangent(0, p, 8, p, p, p, p, None, p, p, 1 << 30, None) == -103
    assert lib.mkpp_gpu_adjoint(4, p, 0, p, p, p, p, p, p, p, 1 << 30, None) == -103
    assert lib.mkpp_gpu_evaluate_rates(0, p, p, p, None) == -103
    assert lib.mkpp_gpu_evaluate_jacobian(4, None, p, p, None) == -101
    h = C.c_void_p()
    assert lib.mkpp_create_handle(C.byref(h), big) == -103

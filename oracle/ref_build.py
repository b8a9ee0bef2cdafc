"""Build the reference's own CPU solver (TEST AND CPU-BASELINE INFRASTRUCTURE ONLY).

Recipe, run where the MKPP reference checkout exists (it is never copied
into the repository):

1. Regenerate the reference's Kokkos C++ solver headers for a mechanism with
   the reference's own compiler pipeline (the steps of ``run_compiler``,
   src/mkpp/cli.py:155-346, called directly), unchanged, with the mechanism plan's tolerances (rtol 1e-3, atol 1 molec/cm3) from an
   environment file, into ``oracle/_ref/gen/<mech>/`` (git-ignored).
2. Compile ``oracle/ref_driver.cpp`` (a small C driver of this project that
   calls the unmodified ``SolverKernels<D>::integrate()`` per cell under
   OpenMP, like the reference's ``RangePolicy(0, cells, ChunkSize(64))``
   dispatch) against those headers and a minimal Kokkos API shim
   (``oracle/kokkos_shim/``, no Kokkos exists on this image) with g++ -O3
   -fopenmp into ``oracle/_ref/libmkpp_ref_<mech>.so``.

The generated headers travel with the repository copy to the GPU machine,
where step 2 runs again (no reference checkout is needed there).  Only tests
and bench.py's CPU-baseline / reference legs load the library.
"""

from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = HERE / "_ref"
GEN = REF / "gen"
MECHS = ("chapman", "small_strato", "saprc99")
# Generated wherever the reference is present but compiled on demand
# (ensure()): TS1's solver takes a minute or more to compile.
ON_DEMAND = ("ts1",)
# Further shipped mechanisms, built on demand by the parity tests (ensure()).
EXTRA_MECHS = ("saprc99_mini", "saprcnov")
# The reference checkout this recipe reads (MKPP_REFERENCE overrides it).
DEFAULT_REFERENCE = os.environ.get("MKPP_REFERENCE", "/root/reference")


# Libraries that are a shipped mechanism with another tableau: name ->
# (mechanism, the reference compiler's solver name).
VARIANTS = {"chapman_rodas3": ("chapman", "rodas3"), "small_strato_rodas3": ("small_strato", "rodas3")}


def _source(lib: str) -> tuple[str, str]:
    """(mechanism, solver) the reference compiler builds library `lib` from."""
    return VARIANTS.get(lib, (lib, "ros3"))


def _tolerances(mech: str) -> tuple[float, float]:
    """(rtol, atol) of the mechanism's plan: the reference solver is
    regenerated at the tolerances the GPU library runs (rtol 1e-3 and atol 1
    molec/cm3, which for TS1's mol/m3 is 1.66e-18)."""
    from mkpp_gb300.emitter.plan import load_raw

    raw = load_raw(mech)
    return float(raw["rtol"][0]), float(raw["atol"][0])


def _yaml_stub():
    if "yaml" in sys.modules:
        return
    try:
        import yaml  # noqa: F401
        return
    except ImportError:
        pass
    m = types.ModuleType("yaml")

    class YAMLError(Exception):
        pass

    m.YAMLError = YAMLError
    m.safe_load = lambda s: json.loads(s.read() if hasattr(s, "read") else s)
    m.dump = m.safe_dump = lambda d, s=None, **k: json.dumps(d)
    sys.modules["yaml"] = m


def generate(mech: str, reference: str = DEFAULT_REFERENCE, host_api: bool = False) -> Path:
    """Step 1: the reference compiler writes gen/<mech>/<mech>.hpp and fragments
    (host_api: host_api/<mech>/ with its generated host API as well: mkpp.h,
    the C++ wrapper mkpp.hpp, the C ABI and the Fortran module)."""
    src, solver = _source(mech)
    out = (REF / "host_api" / mech) if host_api else (GEN / mech)
    if (out / ("mkpp.hpp" if host_api else f"{src}.hpp")).exists():
        return out
    out.mkdir(parents=True, exist_ok=True)
    env = out / "env.json"
    rtol, atol = _tolerances(mech)
    env.write_text(json.dumps({"environment": {"temperature": 298.15, "air_density": 2.46e19},
                               "solver": {"rtol": rtol, "atol": atol}}))
    code = (
        "import sys; sys.dont_write_bytecode = True; "
        f"sys.path.insert(0, {str(HERE.parent)!r}); from oracle.ref_build import _yaml_stub; _yaml_stub(); "
        f"sys.path.insert(0, {reference + '/src'!r}); "
        "from mkpp.parser import load_environment, load_mechanism; "
        "from mkpp.lowering import partition_reactions, prepare_adjoint_and_tlm, prepare_unified_jacobian; "
        "from mkpp.codegen import generate_headers; "
        f"env = load_environment({str(env)!r}); "
        f"mech = load_mechanism({reference + '/mechanisms/openatmos/' + src + '/mechanism.json'!r}); "
        # the metadata wiring of run_compiler (src/mkpp/cli.py:223-236)
        "mech.metadata = mech.metadata or {}; "
        "mech.metadata['temperature'] = str(env.temperature); mech.metadata['air_density'] = str(env.air_density); "
        "mech.metadata['atol'] = [env.solver_atol] * len(mech.species); "
        "mech.metadata['rtol'] = [env.solver_rtol] * len(mech.species); "
        "b = partition_reactions(mech); mech.partition_metadata = b.get('metadata'); "
        "prepare_adjoint_and_tlm(mech); mech.sympy_metadata = prepare_unified_jacobian(mech); "
        f"generate_headers(mech, out_dir={str(out)!r}, solver_name={solver!r}, generate_host_api={host_api!r})"
    )
    subprocess.run([sys.executable, "-c", code], check=True, cwd=str(out),
                   env=dict(os.environ, PYTHONDONTWRITEBYTECODE="1"))
    return out


def lib_path(mech: str) -> Path:
    return REF / f"libmkpp_ref_{mech}.so"


def compile_driver(mech: str) -> Path:
    """Step 2: g++ -O3 -fopenmp the driver against the regenerated headers."""
    base, _ = _source(mech)
    gen = GEN / mech
    out = lib_path(mech)
    src = HERE / "ref_driver.cpp"
    if out.exists() and out.stat().st_mtime >= max(src.stat().st_mtime, (gen / f"{base}.hpp").stat().st_mtime):
        return out
    tmp = out.with_suffix(f".so.tmp{os.getpid()}")
    cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++20", "-fopenmp", "-shared", "-fPIC",
           f"-I{HERE / 'kokkos_shim'}", f"-I{gen}", f"-DMKPP_REF_HEADER=\"{base}.hpp\"",
           f"-DMKPP_REF_NS=mkpp::generated::{base}", str(src), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


def shipped_lib_path(mech: str) -> Path:
    return REF / f"libmkpp_ref_{mech}_shipped.so"


def compile_shipped(mech: str, reference: str = DEFAULT_REFERENCE) -> Path | None:
    """The driver against the reference's shipped generated solver
    (``mkpp-generated/<mech>.hpp``, compiled where it lies, with its own
    tolerances: the build behind the reference's native Kokkos reports).
    None where the reference tree is absent."""
    gen = Path(reference) / "mkpp-generated"
    if not (gen / f"{mech}.hpp").exists():
        return None
    out = shipped_lib_path(mech)
    src = HERE / "ref_driver.cpp"
    if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    REF.mkdir(parents=True, exist_ok=True)
    tmp = out.with_suffix(f".so.tmp{os.getpid()}")
    cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++20", "-fopenmp", "-shared", "-fPIC",
           f"-I{HERE / 'kokkos_shim'}", f"-I{gen}", f"-DMKPP_REF_HEADER=\"{mech}.hpp\"",
           f"-DMKPP_REF_NS=mkpp::generated::{mech}", str(src), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


def ensure(mech: str, reference: str = DEFAULT_REFERENCE):
    """RefSolver for mech, regenerated and compiled first where the reference
    checkout (or headers generated from it earlier) is present; else None."""
    if Path(reference).exists():
        generate(mech, reference)
    if not (GEN / mech / f"{_source(mech)[0]}.hpp").exists():
        return None
    compile_driver(mech)
    return RefSolver(mech)


def build_if_available(reference: str = DEFAULT_REFERENCE) -> list[Path]:
    built = []
    if Path(reference).exists():
        for mech in ON_DEMAND + tuple(VARIANTS):
            generate(mech, reference)
    for mech in MECHS:
        if Path(reference).exists():
            generate(mech, reference)
        if (GEN / mech / f"{mech}.hpp").exists():
            built.append(compile_driver(mech))
    return built


class RefSolver:
    """The reference's generated integrate() on host cores, Oracle-like API."""

    def __init__(self, mech: str, path: Path | None = None):
        from mkpp_gb300.emitter.plan import load_raw

        self.raw = load_raw(mech)
        self.lib = C.CDLL(str(path or lib_path(mech)))
        self.lib.mkpp_ref_integrate.restype = C.c_int
        self.lib.mkpp_ref_num_species.restype = C.c_int
        self.lib.mkpp_ref_num_parameters.restype = C.c_int
        self.ns = self.lib.mkpp_ref_num_species()
        self.np_ = self.lib.mkpp_ref_num_parameters()

    def integrate(self, conc, dt, steps=1, temp=None, rho=None, rh=None, clw=None, param=None, nthreads=0,
                  seed=None, chunk=64, **_):
        conc = np.ascontiguousarray(conc, dtype=np.float64)
        n = conc.shape[1]
        full = lambda a, v: np.ascontiguousarray(np.full(n, v) if a is None else a, dtype=np.float64)  # noqa: E731
        T, RHO, RH, CLW = full(temp, 298.15), full(rho, 2.46e19), full(rh, 0.5), full(clw, 0.0)
        P = np.zeros((max(1, self.np_), n)) if param is None else np.ascontiguousarray(param, dtype=np.float64)
        vp = C.c_void_p
        rc = self.lib.mkpp_ref_integrate(C.c_int(n), vp(conc.ctypes.data), vp(T.ctypes.data), vp(RH.ctypes.data),
                                         vp(CLW.ctypes.data), vp(RHO.ctypes.data), vp(P.ctypes.data),
                                         C.c_int(P.shape[0]),
                                         C.c_double(dt), C.c_int(steps), C.c_int(nthreads),
                                         C.c_double(-1.0 if seed is None else seed), C.c_int(chunk))
        return {"conc": conc, "status": np.zeros(n, np.int32), "rc": rc}

    def evaluate(self, conc, temp=None, rho=None, rh=None, param=None, clw=None, **_):
        """(F [ns][cells], J [ns][ns][cells]) from compute_rates / compute_jacobian."""
        conc = np.ascontiguousarray(conc, dtype=np.float64)
        n = conc.shape[1]
        full = lambda a, v: np.ascontiguousarray(np.full(n, v) if a is None else a, dtype=np.float64)  # noqa: E731
        T, RHO, RH, CLW = full(temp, 298.15), full(rho, 2.46e19), full(rh, 0.5), full(clw, 0.0)
        P = np.zeros((max(1, self.np_), n)) if param is None else np.ascontiguousarray(param, dtype=np.float64)
        F = np.zeros((self.ns, n))
        J = np.zeros((self.ns, self.ns, n))
        vp = C.c_void_p
        args = (C.c_int(n), vp(conc.ctypes.data), vp(T.ctypes.data), vp(RH.ctypes.data), vp(CLW.ctypes.data),
                vp(RHO.ctypes.data), vp(P.ctypes.data), C.c_int(P.shape[0]))
        self.lib.mkpp_ref_rates(*args, vp(F.ctypes.data))
        self.lib.mkpp_ref_jacobian(*args, vp(J.ctypes.data))
        return F, J


def load(mech: str):
    """RefSolver for mech if its library is built here, else None."""
    return RefSolver(mech) if lib_path(mech).exists() else None


if __name__ == "__main__":
    for p in build_if_available():
        print(p)

"""Build the per-mechanism CUDA libraries (sm_103a) in-tree.

Each mechanism library ``mkpp_gb300/lib/libmkpp_<name>.so`` is one nvcc
translation unit: ``csrc/mkpp_capi.cu`` with the generated
``generated/<name>.cuh`` included.  Libraries are rebuilt only when a source
is newer than the library.  Builds run in parallel.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
GEN = PKG / "generated"
LIB = PKG / "lib"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Libraries build() makes by default.  chapman_shipped is Chapman at the
# shipped generated header's tolerances (rtol 1e-6, atol 1e-3), for the
# reference's native-run golden output; chapman_rodas3 and
# small_strato_rodas3 are those mechanisms with the RODAS-3 tableau
# (src/mkpp/rosenbrock.py:71-82) instead of ROS-3.  saprcnov (96 species, as
# large as SAPRC99 to compile, no benchmark configuration) is built on
# request: build(("saprcnov",)).
DEFAULT_MECHANISMS = ("chapman", "small_strato", "saprc99", "ts1", "saprc99_mini", "chapman_shipped",
                      "chapman_rodas3", "small_strato_rodas3")


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mkpp_gb300")


def lib_path(mech: str) -> Path:
    return LIB / f"libmkpp_{mech}.so"


# One translation unit per large kernel instantiation, compiled in parallel:
# the unrolled attempt of a large mechanism takes one to two minutes of
# cicc + ptxas per kernel.  The heaviest units come first.
UNITS = ("mkpp_adjoint.cu", "mkpp_checkpoint.cu", "mkpp_replay.cu", "mkpp_tangent.cu", "mkpp_capi.cu",
         "mkpp_plain.cu", "mkpp_persist4.cu", "mkpp_tail.cu", "mkpp_eval.cu", "mkpp_coop.cu", "mkpp_diff.cu")


# Units of a table-driven mechanism (too large to unroll, such as TS1): its
# unrolled F/J evaluation kernels would take minutes to compile, so its
# evaluation entries walk a table instead (mkpp_eval_table.cu).
UNROLLED_ONLY = ("mkpp_eval.cu",)


def is_table(mech: str) -> bool:
    """True if the mechanism's generated header walks tables instead of
    unrolled code (read from the header, which the emitter writes first)."""
    return "TABLE_ATTEMPT = true" in (GEN / f"{mech}.cuh").read_text()


def units(mech: str) -> tuple[str, ...]:
    if is_table(mech):
        return tuple(u for u in UNITS if u not in UNROLLED_ONLY) + ("mkpp_eval_table.cu",)
    return UNITS


def _sources(mech: str) -> list[Path]:
    return [*(CSRC / u for u in units(mech)), CSRC / "capi_common.cuh", CSRC / "solver.cuh", CSRC / "eval_common.cuh",
            CSRC / "mkpp_device.cuh", GEN / f"{mech}.cuh", INCLUDE / "mkpp.h", Path(__file__)]


def _stale(mech: str) -> bool:
    out = lib_path(mech)
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.exists() and s.stat().st_mtime > t for s in _sources(mech))


def _flags(mech: str, verbose: bool) -> list[str]:
    return [
        *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
        # Only explicit fma() calls fuse: the unrolled and the warp-cooperative
        # attempt then round identically, element by element.
        "--fmad=false",
        "--extended-lambda", "-Xptxas", "-v" if verbose else "-O3",
        f"-DMKPP_MECH_HEADER=\"{mech}.cuh\"", f"-DMKPP_MECH_NS=mkpp_{mech}",
        f"-I{GEN}", f"-I{CSRC}", f"-I{INCLUDE}",
    ]


def _compile_unit(mech: str, unit: str, verbose: bool) -> Path:
    obj = LIB / f"obj_{mech}" / unit.replace(".cu", ".o")
    obj.parent.mkdir(parents=True, exist_ok=True)
    tmp = obj.with_suffix(f".o.tmp{os.getpid()}")
    cmd = [nvcc(), *_flags(mech, verbose), "-c", str(CSRC / unit), "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        tmp.unlink(missing_ok=True)
        raise RuntimeError(f"nvcc failed for {mech}/{unit}:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    if verbose:
        sys.stderr.write(proc.stderr)
    os.replace(tmp, obj)
    return obj


def _link(mech: str, objs: list[Path]) -> Path:
    out = lib_path(mech)
    tmp = out.with_suffix(f".so.tmp{os.getpid()}")
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        tmp.unlink(missing_ok=True)
        raise RuntimeError(f"link failed for {mech}:\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, out)
    return out


def compile_mechanism(mech: str, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile the units of one mechanism in parallel and link the library."""
    LIB.mkdir(parents=True, exist_ok=True)
    us = units(mech)
    with ThreadPoolExecutor(max_workers=len(us)) as ex:
        objs = list(ex.map(lambda u: _compile_unit(mech, u, verbose), us))
    return _link(mech, objs)


def compile_probe() -> Path:
    out = LIB / "libgb300_fp64_probe.so"
    src = CSRC / "probe.cu"
    if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    LIB.mkdir(parents=True, exist_ok=True)
    tmp = out.with_suffix(f".so.tmp{os.getpid()}")
    subprocess.run([nvcc(), *ARCH, "-O3", "-shared", "-Xcompiler", "-fPIC", str(src), "-o", str(tmp)], check=True)
    os.replace(tmp, out)
    return out


def build(mechanisms=DEFAULT_MECHANISMS, force: bool = False, verbose: bool = False, jobs: int | None = None) -> list[Path]:
    from .emitter import cuda_emitter

    for m in mechanisms:
        cuda_emitter.write(m)
    todo = [m for m in mechanisms if force or _stale(m)]
    # Largest translation units first so they overlap the small ones.
    todo.sort(key=lambda m: -(GEN / f"{m}.cuh").stat().st_size)
    with ThreadPoolExecutor(max_workers=jobs or max(1, min(len(todo) + 1, os.cpu_count() or 4))) as ex:
        futs = [ex.submit(compile_mechanism, m, verbose) for m in todo]
        futs.append(ex.submit(compile_probe))
        for f in futs:
            f.result()
    return [lib_path(m) for m in mechanisms]


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("mechanisms", nargs="*", default=list(DEFAULT_MECHANISMS))
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    for p in build(a.mechanisms, force=a.force, verbose=a.verbose):
        print(p)

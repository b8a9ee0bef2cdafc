"""Host builds of the emitted GPU arithmetic (tests/hostsim/).

compile() builds tests/hostsim/attempt_driver.cpp against one generated
header (mkpp_gb300/generated/<m>.cuh).  The CUDA qualifiers become plain C++
(tests/hostsim/cuda_runtime.h), and -ffp-contract=off lets only explicit
fma() calls fuse, as in the GPU build (--fmad=false).  The remaining helpers
run one step of the emitted per-thread code on one cell.
"""

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent


def compile(out_dir, mech, include_first=None):
    """The hostsim library of `mech`; `include_first` is searched for the
    header before mkpp_gb300/generated."""
    out_dir = Path(out_dir)
    so = out_dir / f"hostsim_{mech}_{'table' if include_first else 'unrolled'}.so"
    inc = ([f"-I{include_first}"] if include_first else []) + [f"-I{ROOT / 'mkpp_gb300' / 'generated'}"]
    subprocess.run(["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
                    f"-I{HERE / 'hostsim'}", *inc, f"-I{ROOT / 'mkpp_gb300' / 'csrc'}",
                    f'-DMKPP_MECH_HEADER="{mech}.cuh"', f"-DMKPP_MECH_NS=mkpp_{mech}",
                    str(HERE / "hostsim" / "attempt_driver.cpp"), "-o", str(so)], check=True)
    lib = C.CDLL(str(so))
    lib.hostsim_attempt.restype = C.c_double
    lib.hostsim_attempt.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    lib.hostsim_tlm.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    return lib


def layout(lib):
    v = (C.c_int * 9)()
    lib.hostsim_layout(v)
    return dict(zip(("NSLOTS", "NV", "NR", "NSTAGE", "Y", "K0", "F", "DY", "KT"), list(v)))


def tangent_step(lib, y, k, h, dy, dk):
    """(dy_new, y_new, status) of one step through the emitted tangent
    (attempt() then tlm_step)."""
    L = layout(lib)
    v = (C.c_int * 3)()
    lib.hostsim_tlm_layout(v)
    DYT, DKR, NT = list(v)
    nv = L["NV"]
    S = np.zeros(NT)
    S[L["Y"]:L["Y"] + nv] = y
    S[DYT:DYT + nv] = dy
    S[DKR:DKR + len(dk)] = dk
    st = C.c_int(0)
    kc = np.ascontiguousarray(k, dtype=np.float64)
    lib.hostsim_tlm(S.ctypes.data, kc.ctypes.data, h, C.byref(st))
    return S[DYT:DYT + nv].copy(), y + S[L["DY"]:L["DY"] + nv], st.value

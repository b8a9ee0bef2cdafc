"""The C-ABI library loads and exports every symbol include/mkpp.h declares (no GPU needed)."""
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "mkpp.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|size_t)\s+(mkpp_\w+)\s*\(", text, re.M)))


def test_header_declares_reference_entry_points():
    syms = set(declared_symbols())
    for name in ("mkpp_create_handle", "mkpp_destroy_handle", "mkpp_initialize", "mkpp_integrate",
                 "mkpp_set_state_ptrs", "mkpp_set_rate_parameter_ptrs", "mkpp_set_photolysis_ptrs",
                 "mkpp_evaluate_rates", "mkpp_evaluate_jacobian", "mkpp_get_last_error",
                 "mkpp_get_species_index", "mkpp_get_photolysis_index", "mkpp_set_cloud_water_ptr",
                 "mkpp_set_aerosol_ptrs"):
        assert name in syms


@pytest.mark.parametrize("mech", ["chapman", "ts1"])
def test_library_exports_every_declared_symbol(mech):
    """Unrolled (chapman) and table-driven (ts1) libraries export the whole
    C ABI."""
    from mkpp_gb300 import build
    from mkpp_gb300.api import SIGNATURES

    try:
        lib = build.build((mech,))[0]
    except RuntimeError as e:  # no nvcc
        pytest.skip(str(e))
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(mkpp_\w+)", out))
    missing = set(declared_symbols()) - exported
    assert not missing, missing
    assert {n for n, _, _ in SIGNATURES} == set(declared_symbols())
    # loading resolves every symbol with ctypes (dlopen only; no CUDA call is made)
    from mkpp_gb300 import api

    api.load_library(mech)


def _c_signatures():
    """{name: (return class, [argument classes])} from include/mkpp.h: a
    pointer (or the mkpp_handle_t pointer typedef) is "ptr", else the type."""
    text = (ROOT / "include" / "mkpp.h").read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*(int|size_t)\s+(mkpp_\w+)\s*\(([^)]*)\)\s*;", text, re.M):
        args = []
        for a in (x.strip() for x in m.group(3).split(",")):
            if not a or a == "void":
                continue
            if "*" in a or a.split()[0] == "mkpp_handle_t":
                args.append("ptr")
            else:
                args.append(" ".join(a.replace("const ", "").split()[:-1]))
        out[m.group(2)] = (m.group(1), args)
    return out


def test_reference_fortran_module_binds_the_header():
    """The reference's Fortran module (src/mkpp/templates/host_api/
    mkpp_mod.f90.j2) binds 17 C functions with bind(C); every one exists in
    include/mkpp.h with the same argument count and ABI classes (pointer,
    size_t, int, double) and an int result, so the unchanged module links
    against these libraries.  The interfaces come from the committed fixture
    tests/golden/fortran_bindings.json (tests/golden/make_golden.py)."""
    import json

    fixture = json.loads((ROOT / "tests" / "golden" / "fortran_bindings.json").read_text())
    c = _c_signatures()
    assert len(fixture["functions"]) == 17
    for f in fixture["functions"]:
        assert f["name"] in c, f["name"]
        ret, args = c[f["name"]]
        assert ret == f["returns"] and args == f["args"], (f["name"], args, f["args"])

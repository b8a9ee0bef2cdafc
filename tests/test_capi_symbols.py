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
    """Unrolled (chapman) and table-driven (ts1, whose evaluation entries
    are stubs) libraries export the whole C ABI."""
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

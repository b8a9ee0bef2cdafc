"""Structure of the exported plans against the reference's shipped generated tables."""
import hashlib
import json
from pathlib import Path

import pytest

from mkpp_gb300.emitter import cuda_emitter
from mkpp_gb300.emitter.plan import jacobian_pattern, load, load_raw

GOLD = Path(__file__).resolve().parent / "golden"
MECHS = ["chapman", "small_strato", "saprc99", "ts1", "saprc99_mini", "saprcnov"]


def _tables(raw):
    comp = raw["compact"]
    lower = [list(e) for e in comp["lower"]]
    upper = [list(e) for e in comp["upper"]]
    return {
        "operations": comp["operations"], "products": comp["products"],
        "lower_offsets": comp["lower_offsets"], "upper_offsets": comp["upper_offsets"],
        "diagonal": comp["diagonals"], "lower": lower, "upper": upper,
    }


@pytest.mark.parametrize("mech", MECHS)
def test_lu_schedule_matches_shipped_generated_code(mech):
    """The exported Doolittle schedule is the one in mkpp-generated/<mech>/supernodal_*.hpp."""
    gold = json.loads((GOLD / f"lu_tables_{mech}.json").read_text())
    mine = _tables(load_raw(mech))
    if "sha256" in gold:
        canon = json.dumps(mine, separators=(",", ":"), sort_keys=True)
        assert len(mine["operations"]) == gold["n_operations"]
        assert len(mine["products"]) == gold["n_products"]
        assert hashlib.sha256(canon.encode()).hexdigest() == gold["sha256"]
    else:
        for key in mine:
            assert mine[key] == gold[key], key


@pytest.mark.parametrize("mech", MECHS)
def test_reduced_plan_invariants(mech):
    p = load(mech)
    assert p.n_var + len(p.fixed_phys) == p.n_species
    # mass-action Jacobian pattern == reference W off-diagonal pattern on variable species
    offdiag = {loc for loc in p.w_slots if loc[0] != loc[1]}
    pat = {x for x in jacobian_pattern(p) if x[0] != x[1]}
    assert pat == offdiag
    # every W slot is an LU slot; diagonals present; products reference earlier outputs only
    assert set(p.w_slots) <= set(p.lu_slots)
    written = set()
    for out, w, b, e, dg in p.ops:
        for q in range(b, e):
            a, c = p.products[q]
            assert a in written and c in written
        if dg >= 0:
            assert dg in written
        written.add(out)
    assert written == set(range(len(p.lu_slots)))


@pytest.mark.parametrize("mech", MECHS + ["chapman_shipped", "chapman_rodas3", "small_strato_rodas3"])
def test_generated_header_is_current(mech):
    plan = load(mech)
    text = cuda_emitter.emit_mechanism(plan)
    path = cuda_emitter.GEN_DIR / f"{mech}.cuh"
    assert path.read_text() == text, "regenerate with python -m mkpp_gb300.emitter.cuda_emitter"
    host = cuda_emitter.GEN_DIR / "host_api" / mech / "mkpp.h"
    assert host.read_text() == cuda_emitter.emit_host_header(plan)
    kernels = cuda_emitter.GEN_DIR / "host_api" / mech / f"{mech}.hpp"
    assert kernels.read_text() == cuda_emitter.emit_solver_kernels_header(plan)


def test_noalloc_scratch_size_in_generated_header(tmp_path):
    """MKPP_NOALLOC_SCRATCH_BYTES of each generated host header equals the
    static array the library defines: MKPP_NOALLOC_MAX_CELLS x NSLOTS
    doubles for a tile store, one double for a register store."""
    import re
    import subprocess
    src = tmp_path / "size.c"
    expected = {"saprc99": 1024 * 2226 * 8, "saprcnov": 1024 * 2111 * 8, "ts1": 1024 * 10395 * 8,
                "saprc99_mini": 1024 * 150 * 8, "chapman": 8, "small_strato": 8}
    for mech, want in expected.items():
        nslots = int(re.search(r"static constexpr int NSLOTS = (\d+);",
                               (cuda_emitter.GEN_DIR / f"{mech}.cuh").read_text()).group(1))
        store = 1024 * nslots * 8 if nslots > cuda_emitter.REGISTER_SLOTS else 8
        assert store == want, mech
        src.write_text('#include <stdio.h>\n#include "mkpp.h"\n'
                       'int main(void) { printf("%lld\\n", (long long)(MKPP_NOALLOC_SCRATCH_BYTES)); return 0; }\n')
        exe = tmp_path / f"size_{mech}"
        subprocess.run(["gcc", "-std=c11", "-I", str(cuda_emitter.GEN_DIR / "host_api" / mech),
                        str(src), "-o", str(exe)], check=True)
        assert int(subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout) == want, mech


def test_tableaux_match_reference_coefficients():
    """ROS-3 coefficients as in src/mkpp/rosenbrock.py:40-51 and chapman.hpp:190-191."""
    tab = load_raw("chapman")["tableau"]
    assert tab["name"] == "ROS-3" and tab["stages"] == 3
    assert tab["Gamma"][0] == 0.435866521508459
    assert tab["C"] == [-1.0156171083877703, 4.07599564525377, 9.20767942983308]
    assert tab["M"] == [1.0, 6.1697947043828245, -0.42772256543218573]
    assert tab["NewF"] == [True, True, False]


def test_tolerance_variant_differs_only_in_name_and_tolerances():
    """chapman_shipped is the Chapman plan exported at the shipped header's
    tolerances (mkpp-generated/chapman.hpp: rtol 1e-6, atol 1e-3), the
    settings of the reference's native-run golden output; its emitted
    headers are current."""
    a, b = load_raw("chapman"), load_raw("chapman_shipped")
    assert sorted(k for k in a if a[k] != b[k]) == ["atol", "name", "rtol"]
    assert set(b["rtol"]) == {1e-6} and set(b["atol"]) == {1e-3}
    plan = load("chapman_shipped")
    assert (cuda_emitter.GEN_DIR / "chapman_shipped.cuh").read_text() == cuda_emitter.emit_mechanism(plan)
    assert ((cuda_emitter.GEN_DIR / "host_api" / "chapman_shipped" / "mkpp.h").read_text()
            == cuda_emitter.emit_host_header(plan))
    assert ((cuda_emitter.GEN_DIR / "host_api" / "chapman_shipped" / "chapman_shipped.hpp").read_text()
            == cuda_emitter.emit_solver_kernels_header(plan))

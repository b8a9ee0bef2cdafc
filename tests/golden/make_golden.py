"""Regenerate the golden fixtures of tests/golden/ from the MKPP reference tree.

Reads (never writes) the reference checkout given by --reference and stores
small JSON fixtures, so the tests never need the reference at run time:

* chapman_kokkos_10x60.json  final state of the reference's native Kokkos run
  (reports/native-kokkos-5.1.1/final-mkpp-chapman.stdout.json) and its inputs
  (benchmarks/solver_comparison/runners/mkpp/main.cpp:36-43);
* chapman_scipy_reference.json  SciPy-Radau golden of the reference's
  e2e test (tests/integration/e2e_validation/data/chapman_reference.json);
* lu_tables_<mech>.json  the factorize_plan operation/product tables and the
  solve_plan tables of the shipped generated code
  (mkpp-generated/<mech>/supernodal_{factorize,solve}.hpp);
* chapman_factorization_kat.json  the 13-slot known-answer test of
  tests/integration/supernodal_factorization/test_factorization_parity.cpp;
* ts1_kokkos_2x300.json  final state of the reference's native Kokkos TS1 run
  (reports/native-kokkos-5.1.1/final-mkpp-ts1.stdout.json) and its inputs:
  initial state and 547 rate parameters
  (benchmarks/solver_comparison/runners/mkpp/ts1_binding_data.hpp), the
  two 300 s segments with photolysis slots scaled by 1.0 and 1.05, T and air
  density (runners/mkpp/main.cpp:212-215, 333-344), and the tolerances of
  the shipped generated solver (mkpp-generated/ts1.hpp);
* fortran_bindings.json  the C functions the reference's Fortran module binds
  (src/mkpp/templates/host_api/mkpp_mod.f90.j2, its bind(C) interfaces): name
  and, per argument, how it crosses the ABI (pointer, size_t, int, double);
* ts1_reference_rates.json  F and the nonzero dense Jacobian entries of the
  reference's own generated TS1 solver (compute_rates / compute_jacobian,
  regenerated and compiled by oracle/ref_build.py) at the inputs above,
  with the photolysis slots scaled by 1.0 and by 1.05.

Usage: python tests/golden/make_golden.py --reference <MKPP checkout> [--lu-only]
"""
import argparse
import hashlib
import json
import re
from pathlib import Path

HERE = Path(__file__).resolve().parent
# Mechanisms whose shipped LU tables are pinned; the large ones as a digest.
LU_MECHS = ("chapman", "small_strato", "saprc99", "ts1", "saprc99_mini", "saprcnov")
LU_DIGEST = ("ts1", "saprcnov")


def tables(text: str, name: str):
    m = re.search(name + r"\[\] = \{(.*?)\};", text, re.S)
    body = m.group(1)
    rows = re.findall(r"\{([^{}]*)\}", body)
    if rows:
        return [[int(x) for x in r.replace(" ", "").split(",") if x] for r in rows]
    return [int(x) for x in body.replace(" ", "").replace("\n", "").split(",") if x]


def lu_tables(ref: Path):
    for mech in LU_MECHS:
        fac = (ref / f"mkpp-generated/{mech}/supernodal_factorize.hpp").read_text()
        sol = (ref / f"mkpp-generated/{mech}/supernodal_solve.hpp").read_text()
        out = {
            "source": f"mkpp-generated/{mech}/supernodal_factorize.hpp, supernodal_solve.hpp",
            "operations": tables(fac, "operations"), "products": tables(fac, "products"),
            "lower_offsets": tables(sol, "lower_offsets"), "upper_offsets": tables(sol, "upper_offsets"),
            "diagonal": tables(sol, "diagonal"), "lower": tables(sol, "lower"), "upper": tables(sol, "upper"),
        }
        if mech in LU_DIGEST:
            # Large: keep counts and a digest of the canonical tables only.
            canon = json.dumps({k: v for k, v in out.items() if k != "source"}, separators=(",", ":"), sort_keys=True)
            out = {"source": out["source"], "n_operations": len(out["operations"]), "n_products": len(out["products"]),
                   "sha256": hashlib.sha256(canon.encode()).hexdigest()}
        (HERE / f"lu_tables_{mech}.json").write_text(json.dumps(out, separators=(",", ":")))


def fortran_bindings(ref: Path):
    """The bind(C) interfaces of the Fortran module template, as ABI classes:
    an argument with the VALUE attribute passes its kind by value, any other
    (intent(out) scalars, c_ptr by reference, character arrays) a pointer."""
    text = (ref / "src/mkpp/templates/host_api/mkpp_mod.f90.j2").read_text()
    kinds = {"c_ptr": "ptr", "c_size_t": "size_t", "c_int": "int", "c_double": "double"}
    out = []
    for m in re.finditer(r'function (\w+)\(([^)]*)\) bind\(C, name="(\w+)"\)(.*?)end function', text, re.S):
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        decl = {}
        for line in m.group(4).splitlines():
            km = re.match(r"\s*(type|integer|real|character)\((?:kind=)?(\w+)\)(.*?)::(.*)", line)
            if not km:
                continue
            names = [n.strip().split("(")[0] for n in km.group(4).split(",")]
            by_value = "value" in km.group(3)
            cls = kinds.get(km.group(2), "ptr") if by_value else "ptr"
            for n in names:
                decl[n] = cls
        out.append({"name": m.group(3), "args": [decl[a] for a in args], "returns": "int"})
    (HERE / "fortran_bindings.json").write_text(json.dumps(
        {"source": "src/mkpp/templates/host_api/mkpp_mod.f90.j2", "functions": out}, indent=1))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("--lu-only", action="store_true",
                    help="write the lu_tables_<mech>.json and fortran_bindings.json fixtures only")
    args = ap.parse_args()
    ref = Path(args.reference)
    lu_tables(ref)
    fortran_bindings(ref)
    if args.lu_only:
        return
    run = json.loads((ref / "reports/native-kokkos-5.1.1/final-mkpp-chapman.stdout.json").read_text())
    vals = run["state"]["checkpoints"][0]["values"]
    (HERE / "chapman_kokkos_10x60.json").write_text(json.dumps({
        "source": "reports/native-kokkos-5.1.1/final-mkpp-chapman.stdout.json",
        "tolerances": {"atol": 1e-3, "rtol": 1e-6},
        "dt": 60.0, "steps": 10, "jvals": [1e-12, 1e-4],
        "initial": {"O": 2.5e9, "O2": 5.1e18, "O3": 8.0e11, "M": 2.46e19},
        "final": vals, "elapsed_ms": run["timing"]["elapsed_ms"], "cell_steps": run["timing"]["cell_steps"],
    }, indent=1))
    sci = json.loads((ref / "tests/integration/e2e_validation/data/chapman_reference.json").read_text())
    keep = {k: sci[k] for k in ("species", "initial_conditions", "jvals", "time_span", "scipy_config", "expected_final")}
    keep["source"] = "tests/integration/e2e_validation/data/chapman_reference.json"
    keep["gate"] = {"rtol": 1e-4, "atol": 1.0, "source": "tests/integration/e2e_validation/test_scipy_validation.cpp:246-247"}
    (HERE / "chapman_scipy_reference.json").write_text(json.dumps(keep, indent=1))
    kat = (ref / "tests/integration/supernodal_factorization/test_factorization_parity.cpp").read_text()
    w = [float(x) for x in re.search(r"COMPACT_SIZE> w\{(.*?)\};", kat, re.S).group(1).replace("\n", "").split(",")]
    dense = [float(x) for x in re.search(r"dense_logical_matrix\{(.*?)\};", kat, re.S).group(1).replace("\n", "").split(",")]
    (HERE / "chapman_factorization_kat.json").write_text(json.dumps({
        "source": "tests/integration/supernodal_factorization/test_factorization_parity.cpp",
        "w": w, "rhs": [1.0, 2.0, 3.0, 4.0], "dense_logical": dense, "residual_tol": 1e-12}, indent=1))
    binding = (ref / "benchmarks/solver_comparison/runners/mkpp/ts1_binding_data.hpp").read_text()

    def arr(name, conv):
        body = re.search(name + r"\{(.*?)\};", binding, re.S).group(1)
        return [conv(x.strip()) for x in body.split(",") if x.strip()]

    shipped = (ref / "mkpp-generated/ts1.hpp").read_text()
    tol = {k: float(re.search(k + r"\[NUM_SPECIES\] = \{ *([^,]+),", shipped).group(1)) for k in ("atol", "rtol")}
    run = json.loads((ref / "reports/native-kokkos-5.1.1/final-mkpp-ts1.stdout.json").read_text())
    last = run["state"]["checkpoints"][-1]
    (HERE / "ts1_kokkos_2x300.json").write_text(json.dumps({
        "source": "reports/native-kokkos-5.1.1/final-mkpp-ts1.stdout.json",
        "inputs": "benchmarks/solver_comparison/runners/mkpp/ts1_binding_data.hpp, main.cpp:212-215,333-344",
        "tolerances": tol, "temperature": 287.45, "air_density": 42.393400541636808, "rh": 0.5,
        "segments_s": [300.0, 300.0], "photolysis_slots": 123, "photolysis_scale": [1.0, 1.05],
        "species": arr("species_names", lambda x: x.strip('"')),
        "initial": arr("initial_state", float), "parameters": arr("reaction_parameters", float),
        "final_time_s": last["time_seconds"], "final": last["values"],
    }, separators=(",", ":")))
    import sys

    import numpy as np

    sys.path.insert(0, str(HERE.parent.parent))
    from oracle import ref_build

    ref_build.generate("ts1", str(ref))
    ref_build.compile_driver("ts1")
    solver = ref_build.RefSolver("ts1")
    binding_inputs = json.loads((HERE / "ts1_kokkos_2x300.json").read_text())
    cases = []
    for scale in binding_inputs["photolysis_scale"]:
        P = np.array(binding_inputs["parameters"])[:, None].copy()
        P[:binding_inputs["photolysis_slots"]] *= scale
        conc = np.array(binding_inputs["initial"])[:, None]
        F, J = solver.evaluate(conc, np.array([binding_inputs["temperature"]]),
                               np.array([binding_inputs["air_density"]]), np.array([binding_inputs["rh"]]), P)
        nz = np.argwhere(J[:, :, 0] != 0.0)
        cases.append({"photolysis_scale": scale, "F": F[:, 0].tolist(),
                      "J": [[int(i), int(j), float(J[i, j, 0])] for i, j in nz]})
    (HERE / "ts1_reference_rates.json").write_text(json.dumps({
        "source": "reference compute_rates / compute_jacobian (mkpp-generated/ts1.hpp, regenerated)",
        "inputs": "ts1_kokkos_2x300.json (initial state, parameters, temperature, air density, rh)",
        "cases": cases}, separators=(",", ":")))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()

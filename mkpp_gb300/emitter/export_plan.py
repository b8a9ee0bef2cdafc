"""Export a mechanism's solver plan from the MKPP compiler front end to JSON.

This is the build-time adapter between the MKPP ahead-of-time compiler and the
GB300 CUDA emitter.  It runs the compiler's own parser and symbolic lowering,
unchanged, and records everything the CUDA emitter and the CPU oracle need:

* the physical species order and which species are fixed
  (``parse_mechanism_micm``, ``src/mkpp/parser.py:76-319``);
* the RCM permutation and the row-wise Doolittle LU schedule
  (``SparsityOptimizer`` ``src/mkpp/lowering.py:1116-1242``,
  ``_compute_lu_core`` ``src/mkpp/lowering.py:894-996``) in the compact
  slot form of ``compact_plan`` (``src/mkpp/compact_plan.py:6-70``);
* the per-reaction rate constants, split from the mass-action monomial of the
  reaction flux built by ``_evaluate_reaction_fluxes``
  (``src/mkpp/lowering.py:167-432``).  The rate constant of reaction r is the
  flux divided by the product of its *variable* reactant concentrations, so it
  still carries the fixed-species factors (third bodies such as AIR or M),
  which are constant during one ``integrate()`` call;
* the net stoichiometry of every reaction on every variable species;
* tolerances, the Rosenbrock tableau and the initial-step seed
  (``src/mkpp/template_context.py:283-326``, ``src/mkpp/rosenbrock.py:27-134``).

The symbol substitutions applied to the rate constants are the ones the
reference printer applies before emitting C++ (``src/mkpp/format_eqn.py:130-166``):
``S_a``, ``v_gas`` and the legacy dummy species become 1, ``M_density`` becomes
the per-cell air density (runtime-environment mechanisms) or the compile-time
environment value, and ``Temp`` becomes the per-cell temperature or the
compile-time environment temperature.  Photolysis ``J_n`` and external
``Rate_idx`` symbols address the runtime parameter row (``format_eqn.py:185-191``).

Usage (needs sympy, networkx and the MKPP compiler sources)::

    python -m mkpp_gb300.emitter.export_plan --mkpp-src <MKPP>/src \
        --mechanism <MKPP>/mechanisms/openatmos/saprc99/mechanism.json \
        --rtol 1e-3 --atol 1 --out mkpp_gb300/mechanisms/saprc99.plan.json
"""

from __future__ import annotations

import argparse
import json
import os
import re
import sys
import types
from pathlib import Path

PLAN_FORMAT = 1


def _install_yaml_stub() -> None:
    """The MKPP parser imports PyYAML at module load; JSON inputs never use it."""
    if "yaml" in sys.modules:
        return
    try:
        import yaml  # noqa: F401

        return
    except ImportError:
        pass
    stub = types.ModuleType("yaml")

    class YAMLError(Exception):
        pass

    def safe_load(stream):
        text = stream.read() if hasattr(stream, "read") else stream
        return json.loads(text)

    def dump(data, stream=None, **_kw):
        text = json.dumps(data, indent=2)
        if stream is None:
            return text
        stream.write(text)
        return None

    stub.YAMLError = YAMLError
    stub.safe_load = safe_load
    stub.dump = dump
    stub.safe_dump = dump
    sys.modules["yaml"] = stub


def _c_expr(expr, sp) -> str:
    """Print a SymPy rate-constant expression as a C99 double expression."""
    text = sp.ccode(expr, standard="C99")
    # ccode prints integer powers of symbols as pow(x, 2); keep them exact.
    return text


def _rename(text: str) -> str:
    text = re.sub(r"\bJ_(\d+)\b", r"P[\1]", text)
    text = re.sub(r"\bRate_(\d+)\b", r"P[\1]", text)
    text = re.sub(r"\bFIX_(\d+)\b", r"FIX[\1]", text)
    return text.replace("ENV_T", "T").replace("ENV_RHO", "RHO")


def _env_names(text: str, runtime_env: bool, env_t: float, env_rho: float) -> str:
    """Temperature and air-density names left in a printed rate constant.

    The lowering keeps some rate laws as one opaque symbol whose name is the
    legacy C text (e.g. ``2.45e-12*exp(-1775.0e0/TEMP)``); the reference's
    printer resolves the names inside it (src/mkpp/format_eqn.py:136-164):
    TEMP, temp and Temp are the temperature and M_density the air density,
    per cell with a runtime environment, else the compile-time values."""
    t = "T" if runtime_env else repr(env_t)
    rho = "RHO" if runtime_env else repr(env_rho)
    text = re.sub(r"\b(?:TEMP|temp|Temp)\b", t, text)
    return re.sub(r"\bM_density\b", rho, text)


# Legacy species the reference's printer sets to 1 in every printed
# expression (src/mkpp/format_eqn.py:136-146).
UNIT_SPECIES = ("DummyCH4", "DummyNMVOC", "FixedOH", "FixedCl")


def _check_mass_action(mech) -> None:
    """Refuse mechanisms whose reference tendencies are not k * monomial sums.

    * Equilibrium coupling adds a relaxation flux towards an analytical
      partition model to F (src/mkpp/lowering.py:375-410).
    * A unit species that is a variable species and a reactant: the printer
      substitutes 1 for it after the symbolic Jacobian is taken, so the
      reference's J keeps a column for it that F no longer depends on."""
    if getattr(mech, "equilibrium_reactions", None):
        raise NotImplementedError(f"{mech.name}: equilibrium coupling is not a mass-action tendency")
    for r in mech.reactions:
        names = r.reactants if isinstance(r.reactants, dict) else {x: 1.0 for x in r.reactants}
        unit = [n for n in names if n in UNIT_SPECIES and any(s.name == n and s.role != "fixed" for s in mech.species)]
        if unit:
            raise NotImplementedError(f"{mech.name}: reactant {unit[0]} is printed as 1 after differentiation")


def export(mkpp_src: str, mechanism: str, rtol: float | None, atol: float | None,
           solver: str = "ros3", seed: float | None = None,
           temperature: float = 298.15, air_density: float = 2.46e19) -> dict:
    sys.dont_write_bytecode = True
    sys.path.insert(0, mkpp_src)
    _install_yaml_stub()
    import sympy as sp

    from mkpp.lowering import (
        _evaluate_reaction_fluxes,
        partition_reactions,
        prepare_adjoint_and_tlm,
        prepare_unified_jacobian,
    )
    from mkpp.parser import load_mechanism
    from mkpp.template_context import build_template_context

    mech = load_mechanism(mechanism)
    _check_mass_action(mech)
    if not getattr(mech, "metadata", None):
        mech.metadata = {}
    # Same metadata wiring as run_compiler (src/mkpp/cli.py:223-236).
    mech.metadata["temperature"] = str(temperature)
    mech.metadata["air_density"] = str(air_density)
    if atol is not None:
        mech.metadata["atol"] = [atol] * len(mech.species)
    if rtol is not None:
        mech.metadata["rtol"] = [rtol] * len(mech.species)
    if seed is not None:
        mech.metadata["initial_step_seed"] = seed
    blocks = partition_reactions(mech)
    mech.partition_metadata = blocks.get("metadata")
    prepare_adjoint_and_tlm(mech)
    mech.sympy_metadata = prepare_unified_jacobian(mech)
    ctx = build_template_context(mech, solver, adjoint=True)

    species = [s.name for s in mech.species]
    n = len(species)
    fixed = [s.role == "fixed" for s in mech.species]
    runtime_env = bool(ctx["has_runtime_environment"])
    env_t = float(ctx["environment_temperature"])
    env_rho = float(ctx["environment_air_density"])

    built = _evaluate_reaction_fluxes(mech)
    fluxes = built["reaction_fluxes"]
    csym = {name: sp.Symbol(f"C_{name}", real=True, nonnegative=True) for name in species}

    # Symbol renaming to the C vocabulary used by the emitters.
    subs = {
        sp.Symbol("S_a", real=True, nonnegative=True): sp.Float(1.0),
        sp.Symbol("v_gas", real=True, nonnegative=True): sp.Float(1.0),
    }
    for name in UNIT_SPECIES:
        subs[sp.Symbol(f"C_{name}")] = sp.Float(1.0)
    temp_sym = sp.Symbol("Temp", real=True, nonnegative=True)
    rho_sym = sp.Symbol("M_density", real=True, nonnegative=True)
    env_T = sp.Symbol("ENV_T", real=True)
    env_RHO = sp.Symbol("ENV_RHO", real=True)
    subs[temp_sym] = env_T if runtime_env else sp.Float(env_t)
    subs[rho_sym] = env_RHO if runtime_env else sp.Float(env_rho)
    fixed_syms = {}
    for idx, name in enumerate(species):
        if fixed[idx]:
            fixed_syms[csym[name]] = sp.Symbol(f"FIX_{idx}", real=True)

    reactions = []
    var_index = {name: i for i, name in enumerate(species) if not fixed[i]}
    for r_idx, (r, flux) in enumerate(zip(mech.reactions, fluxes)):
        reactants = r.reactants if isinstance(r.reactants, dict) else {x: 1.0 for x in r.reactants}
        products = r.products if isinstance(r.products, dict) else {x: 1.0 for x in r.products}
        monomial = sp.Integer(1)
        var_reactants = []
        for name, nu in reactants.items():
            if name in var_index:
                power = int(nu)
                monomial *= csym[name] ** sp.Integer(power)
                var_reactants.append([species.index(name), power])
        k_expr = flux / monomial
        leftover = {s for s in k_expr.free_symbols if s.name.startswith("C_") and s.name[2:] in var_index}
        if leftover:
            raise ValueError(f"reaction {r_idx}: rate constant still depends on variable species {leftover}")
        k_expr = k_expr.subs(subs).subs(fixed_syms)
        # Net stoichiometry on variable species, in the order the reference
        # accumulates it (reactants, then products; src/mkpp/lowering.py:389-402).
        net: dict[int, float] = {}
        for name, nu in reactants.items():
            if name in var_index:
                net[species.index(name)] = net.get(species.index(name), 0.0) - float(nu)
        for name, y in products.items():
            if name in var_index:
                net[species.index(name)] = net.get(species.index(name), 0.0) + float(y)
        net_list = [[s, c] for s, c in net.items() if c != 0.0]
        if flux == 0:
            # A rate constant that is identically zero (an Arrhenius A of 0.0)
            # makes the lowered flux 0: the reaction enters neither F nor the
            # Jacobian's sparsity pattern (src/mkpp/lowering.py:167-432).
            var_reactants, net_list = [], []
        text = _env_names(_rename(_c_expr(k_expr, sp)), runtime_env, env_t, env_rho)
        if re.search(r"\bC_\w+", text):
            raise ValueError(f"reaction {r_idx}: unmapped species symbol in rate constant: {text}")
        # Derivatives of the rate constant with respect to fixed species, for
        # the fixed-species columns of the dense Jacobian (compute_jacobian).
        dk = []
        for fsym in sorted(k_expr.free_symbols & set(fixed_syms.values()), key=lambda s: int(s.name[4:])):
            dk.append([int(fsym.name[4:]), _rename(_c_expr(sp.diff(k_expr, fsym), sp))])
        reactions.append({
            "index": r_idx,
            "type": r.reaction_type,
            "k": text,
            "dk_dfixed": dk,
            "reactants": var_reactants,
            "net": net_list,
        })

    compact = ctx["compact"]
    perm = ctx["permutation"] or list(range(n))
    jac_entries = [[int(i), int(j)] for i, j, _ in ctx["jacobian_entries_state"]]
    tab = ctx["tableau"]
    plan = {
        "format": PLAN_FORMAT,
        "name": mech.name,
        "solver": solver,
        "species": species,
        "fixed": fixed,
        "runtime_environment": runtime_env,
        "cloud_gated": bool(ctx["has_cloud_gated"]),
        "environment_temperature": env_t,
        "environment_air_density": env_rho,
        "num_rate_parameters": int(ctx["num_runtime_parameters"]),
        "num_photolysis": int(ctx["num_photolysis"]),
        "photolysis_reactions": [
            {"photo_idx": p["photo_idx"], "reaction_idx": p["reaction_idx"]} for p in ctx["photolysis_reactions"]
        ],
        "num_reactions": len(mech.reactions),
        "atol": [float(x) for x in ctx["tolerance_arrays"]["atol"]],
        "rtol": [float(x) for x in ctx["tolerance_arrays"]["rtol"]],
        "initial_step_seed": float(ctx["initial_step_seed"]),
        "tableau": {
            "name": tab["name"], "stages": tab["stages"], "ELO": tab["ELO"],
            "Gamma": tab["Gamma"], "M": tab["M"], "E": tab["E"], "Alpha": tab["Alpha"],
            "NewF": tab["NewF"], "A": tab["A_matrix"], "C": tab["C_matrix"],
        },
        "permutation": [int(x) for x in perm],
        "jacobian_entries": jac_entries,
        "compact": {
            "w_locations": [list(map(int, loc)) for loc in compact["w_locations"]],
            "j_slot_of_w": [compact["j_slots"].get(tuple(loc), -1) for loc in compact["w_locations"]],
            "lu_locations": [list(map(int, loc)) for loc, _ in sorted(compact["lu_slots"].items(), key=lambda kv: kv[1])],
            "operations": [[o["output"], o["w"], o["begin"], o["end"], o["diagonal"]] for o in compact["operations"]],
            "products": [list(map(int, p)) for p in compact["products"]],
            "lower": [list(map(int, e)) for e in compact["lower"]],
            "upper": [list(map(int, e)) for e in compact["upper"]],
            "lower_offsets": compact["lower_offsets"],
            "upper_offsets": compact["upper_offsets"],
            "diagonals": compact["diagonals"],
        },
        "reactions": reactions,
    }
    return plan


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--mkpp-src", required=True, help="directory holding the mkpp compiler package")
    ap.add_argument("--mechanism", required=True, help="OpenAtmos mechanism JSON")
    ap.add_argument("--out", required=True)
    ap.add_argument("--rtol", type=float, default=None)
    ap.add_argument("--atol", type=float, default=None)
    ap.add_argument("--seed", type=float, default=None)
    ap.add_argument("--solver", default="ros3")
    ap.add_argument("--temperature", type=float, default=298.15)
    ap.add_argument("--air-density", type=float, default=2.46e19)
    ap.add_argument("--name", default=None,
                    help="library name, for a second build of a mechanism (e.g. at other tolerances)")
    args = ap.parse_args(argv)
    os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
    plan = export(args.mkpp_src, args.mechanism, args.rtol, args.atol, args.solver, args.seed,
                  args.temperature, args.air_density)
    if args.name:
        plan["name"] = args.name
    Path(args.out).parent.mkdir(parents=True, exist_ok=True)
    with open(args.out, "w") as f:
        json.dump(plan, f, separators=(",", ":"))
        f.write("\n")
    print(f"{plan['name']}: {len(plan['species'])} species, {len(plan['reactions'])} reactions, "
          f"{len(plan['compact']['lu_locations'])} LU slots -> {args.out}")
    return 0


if __name__ == "__main__":
    sys.exit(main())

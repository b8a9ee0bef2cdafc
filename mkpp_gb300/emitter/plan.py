"""Solver plan model shared by the CUDA emitter, the CPU oracle tables and tests.

A plan JSON (written by ``export_plan.py`` from the MKPP compiler front end)
holds the reference's full N x N structure: physical species order, RCM
permutation, compact W/LU slots and the row-wise Doolittle operation list of
``compact_plan`` (``src/mkpp/compact_plan.py:6-70``).

The GPU kernels work on the *reduced* system that keeps only variable
species.  A fixed species (AIR, M, N2, ...) has an identically zero tendency,
so its Jacobian row is empty (``src/mkpp/lowering.py:389-402`` never
accumulates into a fixed species).  Consequences in the reference's own
factorisation, all exact in IEEE arithmetic:

* its W row is the diagonal ``inv_g_dt`` alone, no L entry ever fills into the
  row, and U holds only the diagonal on that row;
* every stage right-hand side on that row is ``F_fixed + sum(c * K_fixed) = 0``,
  so the forward sweep gives ``y = 0`` and the backward sweep ``K = 0 / U_ii = 0``;
* entries in the fixed species' *column* are only ever multiplied by that zero
  ``y`` or ``K`` (a product ``L(i,f) * U(f,j)`` needs a U entry right of the
  diagonal on row f, and there is none), so ``x - L*0 = x`` leaves every
  variable-species value bit-identical;
* the error-norm contribution of the row is ``(0 / sc)^2 = 0`` while the
  norm still divides by the full species count N (``integrate.j2:265-322``).

Dropping those rows and columns therefore keeps the variable-species LU
values, their product order and the solve order exactly as the reference
computes them.
"""

from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path

MECH_DIR = Path(__file__).resolve().parent.parent / "mechanisms"


@dataclass
class Reaction:
    index: int
    rtype: str
    k: str                        # C expression of the rate constant
    reactants: list[tuple[int, int]]   # (physical variable-species index, power)
    net: list[tuple[int, float]]       # (physical variable-species index, net stoichiometry)


@dataclass
class ReducedPlan:
    """Variable-species system in RCM (logical) order."""

    name: str
    n_species: int                 # N including fixed species (error-norm divisor)
    n_var: int                     # number of variable species
    var_phys: list[int]            # logical variable index -> physical species index
    phys_to_var: dict[int, int]    # physical species index -> logical variable index
    fixed_phys: list[int]          # physical indices of fixed species
    w_slots: list[tuple[int, int]]       # reduced W/LU structure: (row, col) in logical var order
    lu_slots: list[tuple[int, int]]      # LU slots (sorted row-major), logical var order
    lu_index: dict[tuple[int, int], int]
    w_index: dict[tuple[int, int], int]
    ops: list[tuple[int, int, int, int, int]]   # (out, w or -1, begin, end, diag or -1)
    products: list[tuple[int, int]]
    lower: list[list[tuple[int, int]]]    # per row: (col, slot)
    upper: list[list[tuple[int, int]]]    # per row: (col, slot), right of diagonal
    diag: list[int]
    reactions: list[Reaction]
    atol: list[float]             # physical order
    rtol: list[float]
    tableau: dict
    seed: float
    runtime_environment: bool
    cloud_gated: bool
    num_rate_parameters: int
    num_photolysis: int
    raw: dict = field(repr=False, default_factory=dict)

    # --- counts used for the algorithmic-work figures -----------------------
    @property
    def lu_fma(self) -> int:
        return len(self.products)

    @property
    def lu_div(self) -> int:
        return sum(1 for o in self.ops if o[4] >= 0)

    @property
    def solve_entries(self) -> tuple[int, int]:
        return sum(len(r) for r in self.lower), sum(len(r) for r in self.upper)


def load_raw(name_or_path: str | Path) -> dict:
    p = Path(name_or_path)
    if not p.suffix:
        p = MECH_DIR / f"{name_or_path}.plan.json"
    with open(p) as f:
        return json.load(f)


def reduce_plan(raw: dict) -> ReducedPlan:
    species = raw["species"]
    n = len(species)
    fixed = raw["fixed"]
    perm = raw["permutation"]                 # logical -> physical
    comp = raw["compact"]
    lu_loc = [tuple(x) for x in comp["lu_locations"]]
    w_loc = [tuple(x) for x in comp["w_locations"]]
    # Logical full index -> logical variable index
    full_to_var = {}
    var_phys = []
    for logical, phys in enumerate(perm):
        if not fixed[phys]:
            full_to_var[logical] = len(var_phys)
            var_phys.append(phys)
    nv = len(var_phys)

    def keep(loc):
        return loc[0] in full_to_var and loc[1] in full_to_var

    # Reduced LU slots keep the reference's row-major sorted slot order.
    lu_keep = [i for i, loc in enumerate(lu_loc) if keep(loc)]
    lu_map = {old: new for new, old in enumerate(lu_keep)}
    lu_slots = [(full_to_var[lu_loc[i][0]], full_to_var[lu_loc[i][1]]) for i in lu_keep]
    w_keep = [i for i, loc in enumerate(w_loc) if keep(loc)]
    w_map = {old: new for new, old in enumerate(w_keep)}
    w_slots = [(full_to_var[w_loc[i][0]], full_to_var[w_loc[i][1]]) for i in w_keep]

    ops = []
    products = []
    prods_full = comp["products"]
    for out, w, begin, end, dg in comp["operations"]:
        if out not in lu_map:
            continue
        nb = len(products)
        for p in range(begin, end):
            a, b = prods_full[p]
            if a in lu_map and b in lu_map:
                products.append((lu_map[a], lu_map[b]))
            else:
                # A product touching a fixed row/column would mean the fixed row is
                # not empty; the reduction argument above would then be wrong.
                raise ValueError(f"{raw['name']}: product touches a fixed species slot")
        ops.append((lu_map[out], w_map[w] if w >= 0 else -1, nb, len(products),
                    lu_map[dg] if dg >= 0 else -1))
    lu_index = {loc: i for i, loc in enumerate(lu_slots)}
    w_index = {loc: i for i, loc in enumerate(w_slots)}
    lower = [[] for _ in range(nv)]
    upper = [[] for _ in range(nv)]
    for (r, c), s in lu_index.items():
        if c < r:
            lower[r].append((c, s))
        elif c > r:
            upper[r].append((c, s))
    for r in range(nv):
        lower[r].sort()
        upper[r].sort()
    diag = [lu_index[(i, i)] for i in range(nv)]
    reactions = [
        Reaction(r["index"], r["type"], r["k"], [tuple(x) for x in r["reactants"]],
                 [tuple(x) for x in r["net"]])
        for r in raw["reactions"]
    ]
    return ReducedPlan(
        name=raw["name"], n_species=n, n_var=nv, var_phys=var_phys,
        phys_to_var={p: i for i, p in enumerate(var_phys)},
        fixed_phys=[i for i in range(n) if fixed[i]],
        w_slots=w_slots, lu_slots=lu_slots, lu_index=lu_index, w_index=w_index,
        ops=ops, products=products, lower=lower, upper=upper, diag=diag,
        reactions=reactions, atol=raw["atol"], rtol=raw["rtol"], tableau=raw["tableau"],
        seed=raw["initial_step_seed"], runtime_environment=raw["runtime_environment"],
        cloud_gated=raw["cloud_gated"], num_rate_parameters=raw["num_rate_parameters"],
        num_photolysis=raw["num_photolysis"], raw=raw,
    )


def load(name: str) -> ReducedPlan:
    return reduce_plan(load_raw(name))


def jacobian_pattern(plan: ReducedPlan) -> set[tuple[int, int]]:
    """Structural (row, col) pattern, logical variable order, of the mass-action J."""
    pat = set()
    for r in plan.reactions:
        for s, _c in r.net:
            for j, _p in r.reactants:
                pat.add((plan.phys_to_var[s], plan.phys_to_var[j]))
    return pat


def flops_per_attempt(plan: ReducedPlan) -> dict[str, int]:
    """Algorithmic FP64 operations of one Rosenbrock attempt on the reduced system.

    Counted per term of the emitted arithmetic (a fused multiply-add is two
    operations; a division, reciprocal, square or cube root is one):
    Jacobian partials and W assembly, LU products (2 each), pivot reciprocals
    and L scalings, each stage's forward/backward sweep (2 per L/U entry plus
    the pivot scaling), the tendency evaluations of the stages with NewF, the
    stage combinations and the error norm.
    """
    tab = plan.tableau
    st = int(tab["stages"])
    nv = plan.n_var
    fun = sum(sum(pw for _, pw in r.reactants) for r in plan.reactions) + \
        sum(2 * len(r.net) for r in plan.reactions)
    jac = sum(2 * len(r.net) * len(r.reactants) for r in plan.reactions) + \
        sum(len(r.reactants) * max(0, sum(pw for _, pw in r.reactants) - 1) for r in plan.reactions) + nv
    lu = 2 * plan.lu_fma + plan.lu_div + nv
    low, up = plan.solve_entries
    solve = 2 * (low + up) + nv
    n_newf = sum(1 for x in tab["NewF"] if x)
    a_terms = sum(1 for i in range(1, st) for j in range(i) if tab["A"][i * (i - 1) // 2 + j] != 0.0 and tab["NewF"][i])
    c_terms = sum(1 for i in range(1, st) for j in range(i) if tab["C"][i * (i - 1) // 2 + j] != 0.0)
    stage = nv * (a_terms + 2 * c_terms) + c_terms
    err = nv * (2 * st + 2 * st + 6) + 3
    total = jac + lu + n_newf * fun + st * solve + stage + err
    return {"jacobian": jac, "lu": lu, "fun": n_newf * fun, "solve": st * solve, "stage": stage, "error": err,
            "total": total}

"""CUDA (sm_103a) emitter: plan JSON -> per-mechanism device header.

The emitted header defines ``struct Mech`` in ``namespace mkpp_<name>`` with
the per-cell arithmetic of one Rosenbrock attempt, fully unrolled, in FP64:

* ``rate_constants``  - the reaction rate constants k_r(T, rho, fixed species,
  runtime parameters), evaluated once per cell and host step instead of inside
  every F/J expression (the reference inlines them,
  ``src/mkpp/templates/device_impl/rates.hpp.j2:9-35``);
* ``fun``             - mass-action F_i = sum_r net_ir * k_r * prod C^nu;
* ``jac_w``           - W = I/(gamma h) - J written straight into the LU slots
  (``integrate.j2:103-107``), J from the per-reaction partial derivatives;
* ``factor``          - the row-wise Doolittle schedule of ``compact_plan``
  (``src/mkpp/compact_plan.py:30-47``, executed by
  ``device_impl/supernodal_factorize.hpp.j2:10-31``) unrolled with constant
  slot indices, in place; each pivot is inverted once and the L entries of its
  column are scaled by the reciprocal;
* ``solve``           - forward (unit L) and backward substitution in the
  order of ``device_impl/supernodal_solve.hpp.j2:10-42``;
* ``attempt``         - the tableau stages, the increment sum M.K and the WRMS
  error norm of ``integrate.j2:144-322``.

The step controller and the kernels that drive it are mechanism independent
and live in ``csrc/solver.cuh``.
"""

from __future__ import annotations

import re
from pathlib import Path

from . import warp_schedule
from .plan import ReducedPlan, load

GEN_DIR = Path(__file__).resolve().parent.parent / "generated"


def _lit(x: float) -> str:
    """Exact C literal for a double (17 significant digits, like ``%.17g``)."""
    s = "%.17g" % float(x)
    if "e" not in s and "." not in s and "n" not in s:
        s += ".0"
    return s


def _k_text(expr: str) -> str:
    expr = re.sub(r"\bP\[(\d+)\]", r"P(\1)", expr)
    expr = re.sub(r"\bFIX\[(\d+)\]", r"FIX(\1)", expr)
    return expr


class _Code:
    def __init__(self):
        self.lines: list[str] = []

    def __call__(self, s: str = ""):
        self.lines.append(s)

    def text(self) -> str:
        return "\n".join(self.lines) + "\n"


def _accumulate(target: str, init: str | None, terms: list[tuple[float, str]]) -> str:
    """Sum ``init + c1*t1 + c2*t2 ...`` left to right, exact signs for +-1."""
    expr = init
    for c, t in terms:
        if expr is None:
            if c == 1.0:
                expr = t
            elif c == -1.0:
                expr = f"-{t}"
            else:
                expr = f"{_lit(c)} * {t}"
            continue
        if c == 1.0:
            expr = f"{expr} + {t}"
        elif c == -1.0:
            expr = f"{expr} - {t}"
        else:
            expr = f"fma({_lit(c)}, {t}, {expr})"
    if expr is None:
        expr = "0.0"
    return f"{target} = {expr};"


def _sum_expr(init: str | None, terms: list[tuple[float, str]]) -> str:
    """Expression ``init + c1*t1 + c2*t2 ...`` accumulated left to right."""
    return _accumulate("@", init, terms)[4:-1]


ILP_GROUP = 8
# Slot count above which the solver keeps a cell's working set in the global
# tile rather than registers (kRegisterSlots in csrc/solver.cuh).
REGISTER_SLOTS = 96


def _interleave(c, plan, ops, operands, scale):
    """Emit the dot products of independent LU ops in interleaved rounds.

    ops are (out, w, begin, end, diag) with disjoint outputs that read only
    values finished earlier.  Groups of ILP_GROUP ops advance one product per
    round, which keeps each op's subtraction order (and so its rounding)
    exactly that of the sequential schedule.
    """
    for g in range(0, len(ops), ILP_GROUP):
        grp = ops[g:g + ILP_GROUP]
        for out, w, b, e, dg in grp:
            c(f"      double v{out} = {'S[%d]' % out if w >= 0 else '0.0'};")
        longest = max(e - b for _, _, b, e, _ in grp)
        for t in range(longest):
            for out, w, b, e, dg in grp:
                if b + t < e:
                    x, y = operands(b + t)
                    c(f"      v{out} = fma(-{x}, {y}, v{out});")
        for out, w, b, e, dg in grp:
            if scale:
                c(f"      S[{out}] = v{out} * {scale};")
            elif not (w >= 0 and e == b):
                c(f"      S[{out}] = v{out};")


def _c_array(c, ctype, name, values):
    vals = list(values) or [0]
    body = ", ".join(str(v) for v in vals)
    c(f"static __device__ const {ctype} {name}[{len(vals)}] = {{{body}}};")


def _c_u64_array(c, name, values):
    vals = list(values) or [0]
    rows = [", ".join(f"0x{v:x}ull" for v in vals[i:i + 8]) for i in range(0, len(vals), 8)]
    c(f"static __device__ const unsigned long long {name}[{len(vals)}] = {{")
    for r in rows:
        c(f"    {r},")
    c("};")


def _coop_build(plan, nv, stages, A, C, NewF, K0, Y, FS, DY, nslots, table=False, M=None):
    """The stage programs of one attempt and the slot layout they use.

    Each tableau stage of the attempt is one program of uniform operations
    (``warp_schedule``), with the per-thread kernel's arithmetic, operation
    by operation, in its order.  Slots beyond the per-thread layout (nslots):
    the rates q_r, the Jacobian partials, and constants (-0, +0, 1,
    1/(gamma h), c_ij/h, literals)."""
    v2l = plan.phys_to_var
    nr = len(plan.reactions)
    nq = max(nr, nv)
    npart = sum(len(r.reactants) for r in plan.reactions)
    Q = nslots                      # rates q_r (then q_i of the error norm)
    D = nslots + nq                 # Jacobian partial derivatives
    CB = D + npart                  # constants: -0, +0, 1, 1/(gamma h), c_ij/h, literals
    adj = None
    if table:
        # The table-driven adjoint's slots sit before the constants: lambda,
        # the stage adjoints, the pending tendency adjoint, dL/dk, and
        # temporaries (one per reaction, one per species, a few scalars).
        adj = {"LAM": CB}
        adj["KBAR"] = adj["LAM"] + nv
        adj["FBAR"] = adj["KBAR"] + stages * nv
        adj["KB"] = adj["FBAR"] + nv
        adj["TMP"] = adj["KB"] + nr
        CB = adj["TMP"] + nr + nv + 8
    ZN, ZP, ONE, IG = CB, CB + 1, CB + 2, CB + 3
    cterm_slot = {}
    for st in range(2, stages + 1):
        for j in range(1, st):
            cv = C[(st - 1) * (st - 2) // 2 + j - 1]
            if cv != 0.0:
                cterm_slot[(st, j)] = CB + 4 + len(cterm_slot)
    literals: dict[float, int] = {}
    lit_base = CB + 4 + len(cterm_slot)

    def lit(v):
        v = float(v)
        if v not in literals:
            literals[v] = lit_base + len(literals)
        return literals[v]

    def program():
        return warp_schedule.Program(ZN, ZP, ONE, lit)

    def fun(P, yv):
        """F(y) into S[FS..] for y in S[yv..]: rates q_r = k_r * y ... in
        reactant order, then F_i as the sum over reactions in reaction order."""
        for r in plan.reactions:
            fac = [v2l[s_] for s_, pw in r.reactants for _ in range(pw)]
            if not fac:
                P.copy(Q + r.index, Mech_KT + r.index)
            for n_, f in enumerate(fac):
                P.mul(Q + r.index, (Mech_KT + r.index) if n_ == 0 else Q + r.index, yv + f)
        contrib = {i: [] for i in range(nv)}
        for r in plan.reactions:
            for s_, coef in r.net:
                contrib[v2l[s_]].append((coef, r.index))
        for i in range(nv):
            if not contrib[i]:
                P.zero(FS + i)
            for n_, (coef, ri) in enumerate(contrib[i]):
                P.acc_term(FS + i, n_ == 0, float(coef), Q + ri)

    def jac_w(P):
        """Partials d = k [* power] * y ... at S[Y..], then W = I/(gamma h) - J
        into the LU slots, and the fill-in slots zeroed."""
        pidx = {}
        p = 0
        for r in plan.reactions:
            terms = list(r.reactants)
            for idx, (s_, pw) in enumerate(terms):
                fac = []
                for jdx, (s2, pw2) in enumerate(terms):
                    if jdx == idx:
                        if pw2 > 1:
                            fac.append(lit(float(pw2)))
                            fac += [Y + v2l[s2]] * (pw2 - 1)
                    else:
                        fac += [Y + v2l[s2]] * pw2
                if not fac:
                    P.copy(D + p, Mech_KT + r.index)
                for n_, f in enumerate(fac):
                    P.mul(D + p, (Mech_KT + r.index) if n_ == 0 else D + p, f)
                pidx[(r.index, s_)] = p
                p += 1
        wterms = {loc: [] for loc in plan.w_slots}
        for r in plan.reactions:
            for s_, coef in r.net:
                for s2, _pw in r.reactants:
                    wterms[(v2l[s_], v2l[s2])].append((-coef, pidx[(r.index, s2)]))
        for loc in plan.w_slots:
            out = plan.lu_index[loc]
            terms = wterms[loc]
            if loc[0] == loc[1]:
                if not terms:
                    P.copy(out, IG)
                for n_, (coef, pi) in enumerate(terms):
                    P.acc_term(out, False, float(coef), D + pi, acc=IG if n_ == 0 else None)
            else:
                if not terms:
                    P.zero(out)
                for n_, (coef, pi) in enumerate(terms):
                    P.acc_term(out, n_ == 0, float(coef), D + pi)
        for sl in warp_schedule.lu_zero_slots(plan):
            P.zero(sl)

    # The rate constants of the host step sit in the KT slots (after the stage
    # vectors, F and the increment): KT = DY + NV.
    Mech_KT = DY + nv
    progs = []
    for st in range(1, stages + 1):
        P = program()
        kb = K0 + (st - 1) * nv
        if st == 1:
            jac_w(P)
            P.lu(plan)
        if NewF[st - 1]:
            if st == 1:
                fun(P, Y)
            else:
                # Stage state Y + sum a_j K_j into the DY slots; Q holds a*K
                # partial terms (rates are written after the state is read).
                terms = []
                for j in range(1, st):
                    a = A[(st - 1) * (st - 2) // 2 + j - 1]
                    if a != 0.0:
                        terms.append((a, j))
                for i in range(nv):
                    acc = Y + i
                    for a, j in terms:
                        kk = K0 + (j - 1) * nv + i
                        if a == 1.0:
                            P.fma(DY + i, kk, ONE, acc)
                        else:
                            P.mul(Q + i, kk, lit(a))
                            P.fma(DY + i, Q + i, ONE, acc)
                        acc = DY + i
                    if not terms:
                        P.copy(DY + i, Y + i)
                fun(P, DY)
        for i in range(nv):
            P.copy(kb + i, FS + i)
            for j in range(1, st):
                if (st, j) in cterm_slot:
                    P.fma(kb + i, cterm_slot[(st, j)], K0 + (j - 1) * nv + i, kb + i)
        P.solve(plan, kb)
        progs.append(P.ops)
    sched = [warp_schedule.schedule(ops) for ops in progs]
    adj_ops = eval_ops = None
    if table:
        P = program()
        _adjoint_program(plan, P, nv, stages, A, C, M, NewF, K0, Y, Mech_KT, adj, cterm_slot)
        adj_ops = P.ops
        # The evaluation entries: W with 1/(gamma h) = 0 (that is -J on the W
        # slots) and F(y) into S[FS..], the first stage's code without the LU.
        P = program()
        jac_w(P)
        fun(P, Y)
        eval_ops = P.ops
        assert all(op[0] != warp_schedule.RCP for op in eval_ops)
    nconst = 4 + len(cterm_slot) + len(literals)
    const_vals = ["-0.0", "0.0", "1.0", "0.0"] + ["0.0"] * len(cterm_slot) + [_lit(v) for v in literals]
    return {"progs": progs, "sched": sched, "npart": npart, "nq": nq, "Q": Q, "D": D, "CB": CB,
            "nconst": nconst, "const_vals": const_vals, "literals": literals, "cterm_slot": cterm_slot,
            "KT": Mech_KT, "total": CB + nconst, "adj": adj, "adj_ops": adj_ops, "eval_ops": eval_ops,
            "A": A, "NewF": NewF}


def _adjoint_program(plan, P, nv, stages, A, C, M, NewF, K0, Y, KT, adj, cterm_slot):
    """The reverse of one accepted step as a sequential program: operation
    for operation the arithmetic of the unrolled ``adjoint_step``
    (``_emit_adjoint``), the same sums in the same order.  A term is a
    product of factors evaluated left to right; a first term with a
    coefficient c other than +-1 is c * f1 * f2 ... (c multiplied in first),
    as the unrolled expressions associate."""
    v2l = plan.phys_to_var
    nr = len(plan.reactions)
    LAM, KBAR, FBAR, KB, TMP = adj["LAM"], adj["KBAR"], adj["FBAR"], adj["KB"], adj["TMP"]
    TS, TY = TMP, TMP + nr                       # per-reaction s, per-species stage state
    T_S, T_G, T_KS, T_H, T_M, T_T, T_X = (TMP + nr + nv + i for i in range(7))

    def product(dest, factors):
        """dest = f1 * f2 * ... left to right (one factor: a copy)."""
        if len(factors) == 1:
            P.copy(dest, factors[0])
            return
        P.mul(dest, factors[0], factors[1])
        for f in factors[2:]:
            P.mul(dest, dest, f)

    def mono(expo, ybase):
        """Slot of prod y^e: the product is formed in T_M if it has more than
        one factor.  Called just before the term that uses it."""
        fac = [ybase(q) for q in sorted(expo) for _ in range(expo[q])]
        if len(fac) == 1:
            return fac[0]
        product(T_M, fac)
        return T_M

    def accumulate(dest, terms):
        """dest = sum over (coef, make) of coef * product(make()): first term
        t, -t or c * f1 * f2 ..., then acc + t, acc - t or fma(c, t, acc)."""
        for n_, (coef, make) in enumerate(terms):
            factors = make()
            if n_ == 0:
                if coef == 1.0:
                    product(dest, factors)
                elif coef == -1.0:
                    product(T_T, factors)
                    P.fma(dest, T_T, P.one, P.zn, neg=True)
                else:
                    product(dest, [P.lit(coef)] + factors)
            else:
                product(T_T, factors)
                if coef == 1.0:
                    P.fma(dest, T_T, P.one, dest)
                elif coef == -1.0:
                    P.fma(dest, T_T, P.one, dest, neg=True)
                else:
                    P.fma(dest, P.lit(coef), T_T, dest)

    def dot(net, base):
        return [(float(co), (lambda i=i: [base + i])) for i, co in net]

    def ymono_v(e2, vslot):
        return lambda: ([mono(e2, lambda q: Y + q), vslot] if e2 else [vslot])

    rx = [(r.index, _monomial_terms(r.reactants, v2l), [(v2l[s_], co) for s_, co in r.net]) for r in plan.reactions]
    ucol = [[] for _ in range(nv)]
    lcol = [[] for _ in range(nv)]
    for (r_, cc), sl in plan.lu_index.items():
        if r_ < cc:
            ucol[cc].append((r_, sl))
        elif r_ > cc:
            lcol[cc].append((r_, sl))

    def solve_t(base):
        """W^T x = b in place: U^T forward (times 1/U_ii), then L^T backward."""
        for i in range(nv):
            for k_, sl in sorted(ucol[i]):
                P.fma(base + i, sl, base + k_, base + i, neg=True)
            P.mul(base + i, base + i, plan.diag[i])
        for i in range(nv - 1, -1, -1):
            for k_, sl in sorted(lcol[i]):
                P.fma(base + i, sl, base + k_, base + i, neg=True)

    def wterm(ub, vb):
        """u^T J(y_n) v terms: dk into KB, Hessian-vector into LAM."""
        for ri, expo, net in rx:
            if not net or not expo:
                continue
            accumulate(T_S, dot(net, ub))
            gterms = []
            for j in sorted(expo):
                coef, e2 = _dmono(expo, j)
                gterms.append((coef, ymono_v(e2, vb + j)))
            accumulate(T_G, gterms)
            P.fma(KB + ri, T_S, T_G, KB + ri)
            P.mul(T_KS, KT + ri, T_S)
            for p_ in sorted(expo):
                c1, e1 = _dmono(expo, p_)
                hterms = []
                for q in sorted(e1):
                    c2, e2 = _dmono(e1, q)
                    hterms.append((c1 * c2, ymono_v(e2, vb + q)))
                if hterms:
                    accumulate(T_H, hterms)
                    P.fma(LAM + p_, T_KS, T_H, LAM + p_)

    def fterm(yslot, aterms):
        """Adjoint of F at the stage state: dk into KB, J^T Fbar into LAM and
        the stage adjoints of the K_j the state is built from."""
        for ri, expo, net in rx:
            if not net:
                continue
            accumulate(TS + ri, dot(net, FBAR))
            if expo:
                P.fma(KB + ri, TS + ri, mono(expo, yslot), KB + ri)
            else:
                P.fma(KB + ri, TS + ri, P.one, KB + ri)
        yb_terms = {j: [] for j in range(nv)}
        for ri, expo, net in rx:
            if not net:
                continue
            for j in sorted(expo):
                coef, e2 = _dmono(expo, j)
                fac = [KT + ri, TS + ri] + [yslot(q) for q in sorted(e2) for _ in range(e2[q])]
                yb_terms[j].append((coef, (lambda fac=fac: fac)))
        for j in range(nv):
            if yb_terms[j]:
                accumulate(T_X, yb_terms[j])
                P.fma(LAM + j, T_X, P.one, LAM + j)
                for a, jj in aterms:
                    P.fma(KBAR + jj * nv + j, P.lit(a), T_X, KBAR + jj * nv + j)

    for i in range(stages):
        for j in range(nv):
            if M[i] != 0.0:
                P.mul(KBAR + i * nv + j, P.lit(M[i]), LAM + j)
            else:
                P.zero(KBAR + i * nv + j)
    for j in range(nv):
        P.zero(FBAR + j)
    used = sorted({j for _, e, _ in rx for j in e})
    for i in range(stages - 1, -1, -1):
        kb = KBAR + i * nv
        solve_t(kb)
        wterm(kb, K0 + i * nv)
        for j in range(nv):
            P.fma(FBAR + j, kb + j, P.one, FBAR + j)
        for j in range(i):
            cv = C[i * (i - 1) // 2 + j]
            if cv != 0.0:
                slot = cterm_slot[(i + 1, j + 1)]
                for q in range(nv):
                    P.fma(KBAR + j * nv + q, slot, kb + q, KBAR + j * nv + q)
        if NewF[i]:
            aterms = [(A[i * (i - 1) // 2 + j], j) for j in range(i) if i > 0 and A[i * (i - 1) // 2 + j] != 0.0]
            if aterms:
                for q in used:
                    acc = Y + q
                    for a, j in aterms:
                        kk = K0 + j * nv + q
                        if a == 1.0:
                            P.fma(TY + q, kk, P.one, acc)
                        else:
                            P.mul(T_T, kk, P.lit(a))
                            P.fma(TY + q, T_T, P.one, acc)
                        acc = TY + q
                fterm(lambda q: TY + q, aterms)
            else:
                fterm(lambda q: Y + q, aterms)
            for j in range(nv):
                P.zero(FBAR + j)


def _tlm_build(plan, nv, stages, A, C, M, NewF, K0, Y, KT, base):
    """Tangent of one accepted step of size h (forward mode), as a sequential
    program of uniform operations with its own slots and constants from
    `base` on.  With W = I/(gamma h) - J(y) and F_i = f(Y_i):
        dY_i = dy + sum_j a_ij dK_j
        dF_i = J(Y_i) dY_i + sum_r net_r dk_r m_r(Y_i)       (NewF stages)
        W dK_i = dF_i + sum_j c_ij/h dK_j + dJ K_i,
        dJ K_i = sum_r net_r (dk_r grad m_r(y).K_i + k_r K_i^T H_r(y) dy)
        dy_new = dy + sum_i M_i dK_i.
    In: dy in DYT, dk in DKR (the rate constants' tangent); out: dy_new in
    DYT.  The LU and the K_i are those attempt() left for this step."""
    v2l = plan.phys_to_var
    nr = len(plan.reactions)
    L = {"DYT": base}
    L["DKR"] = L["DYT"] + nv
    L["DK"] = L["DKR"] + nr
    L["DF"] = L["DK"] + stages * nv
    L["TY"] = L["DF"] + nv
    L["TD"] = L["TY"] + nv
    TT = L["TD"] + nv
    TCB = TT + 8
    L["TCB"] = TCB
    DYT, DKR, DK, DF, TY, TD = L["DYT"], L["DKR"], L["DK"], L["DF"], L["TY"], L["TD"]
    T_A, T_B, T_P = TT, TT + 1, TT + 2
    cterm = {}
    for st in range(2, stages + 1):
        for j in range(1, st):
            if C[(st - 1) * (st - 2) // 2 + j - 1] != 0.0:
                cterm[(st, j)] = TCB + 3 + len(cterm)
    literals: dict[float, int] = {}
    lit_base = TCB + 3 + len(cterm)

    def lit(v):
        v = float(v)
        if v not in literals:
            literals[v] = lit_base + len(literals)
        return literals[v]

    P = warp_schedule.Program(TCB, TCB + 1, TCB + 2, lit)

    def product(dest, factors):
        if not factors:
            P.copy(dest, P.one)
        elif len(factors) == 1:
            P.copy(dest, factors[0])
        else:
            P.mul(dest, factors[0], factors[1])
            for f in factors[2:]:
                P.mul(dest, dest, f)

    def add_scaled(dest, coef, src):
        if coef == 1.0:
            P.fma(dest, src, P.one, dest)
        elif coef == -1.0:
            P.fma(dest, src, P.one, dest, neg=True)
        else:
            P.fma(dest, lit(coef), src, dest)

    def ys_of(expo, yslot):
        return [yslot(q) for q in sorted(expo) for _ in range(expo[q])]

    def grad_dot(dest, expo, yslot, vslot):
        """dest = sum_j dm/dy_j (y) v_j"""
        P.zero(dest)
        for j in sorted(expo):
            c1, e2 = _dmono(expo, j)
            product(T_P, ys_of(e2, yslot) + [vslot(j)])
            add_scaled(dest, c1, T_P)

    def hess(dest, expo, yslot, uslot, vslot):
        """dest = sum_p sum_q u_p d2m/dy_p dy_q (y) v_q"""
        P.zero(dest)
        for p_ in sorted(expo):
            c1, e1 = _dmono(expo, p_)
            for q in sorted(e1):
                c2, e2 = _dmono(e1, q)
                product(T_P, ys_of(e2, yslot) + [uslot(p_), vslot(q)])
                add_scaled(dest, c1 * c2, T_P)

    rx = [(r.index, _monomial_terms(r.reactants, v2l), [(v2l[s_], co) for s_, co in r.net]) for r in plan.reactions]
    for i in range(stages):
        kb = DK + i * nv
        if NewF[i]:
            aterms = [(A[i * (i - 1) // 2 + j], j) for j in range(i) if i > 0 and A[i * (i - 1) // 2 + j] != 0.0]
            if aterms:
                for q in range(nv):
                    P.copy(TY + q, Y + q)
                    P.copy(TD + q, DYT + q)
                    for a_, j in aterms:
                        add_scaled(TY + q, a_, K0 + j * nv + q)
                        add_scaled(TD + q, a_, DK + j * nv + q)
                ys, ds = (lambda q: TY + q), (lambda q: TD + q)
            else:
                ys, ds = (lambda q: Y + q), (lambda q: DYT + q)
            for q in range(nv):
                P.zero(DF + q)
            for ri, expo, net in rx:
                if not net:
                    continue
                if expo:
                    grad_dot(T_A, expo, ys, ds)
                    P.mul(T_A, KT + ri, T_A)
                else:
                    P.zero(T_A)
                product(T_B, ys_of(expo, ys))
                P.fma(T_A, DKR + ri, T_B, T_A)
                for p_, co in net:
                    add_scaled(DF + p_, float(co), T_A)
        for q in range(nv):
            P.copy(kb + q, DF + q)
            for j in range(i):
                if (i + 1, j + 1) in cterm:
                    P.fma(kb + q, cterm[(i + 1, j + 1)], DK + j * nv + q, kb + q)
        for ri, expo, net in rx:
            if not net or not expo:
                continue
            grad_dot(T_A, expo, lambda q: Y + q, lambda q, i=i: K0 + i * nv + q)
            P.mul(T_A, DKR + ri, T_A)
            hess(T_B, expo, lambda q: Y + q, lambda p_, i=i: K0 + i * nv + p_, lambda q: DYT + q)
            P.fma(T_A, KT + ri, T_B, T_A)
            for p_, co in net:
                add_scaled(kb + p_, float(co), T_A)
        P.solve(plan, kb)
    for q in range(nv):
        for i in range(stages):
            if M[i] != 0.0:
                add_scaled(DYT + q, M[i], DK + i * nv + q)
    nconst = 3 + len(cterm) + len(literals)
    const_vals = ["-0.0", "0.0", "1.0"] + ["0.0"] * len(cterm) + [_lit(v) for v in literals]
    return {"ops": P.ops, "L": L, "cterm": cterm, "nconst": nconst, "const_vals": const_vals,
            "total": TCB + nconst}


def _emit_tlm(c, t, tlm, C):
    """Constants, tables (into the coop namespace text t) and tlm_step."""
    L = tlm["L"]
    ops = tlm["ops"]
    t(f"constexpr int TLM_OPS = {len(ops)};")
    t(f"static __device__ const double tlm_const_val[{tlm['nconst']}] = {{{', '.join(tlm['const_vals'])}}};")
    _c_u64_array(t, "tlm_prog", warp_schedule.encode(ops, [[i] for i in range(len(ops))], lanes=1))
    c("")
    c("  // ---- tangent of one accepted step (forward sensitivities) ----")
    c(f"  static constexpr int DYT = {L['DYT']};     // dy in, dy_new out (NV)")
    c(f"  static constexpr int DKR = {L['DKR']};     // dk, the rate constants' tangent (NR)")
    c(f"  static constexpr int TLM_CB = {L['TCB']};  // constants of the tangent program")
    c(f"  static constexpr int TLM_NCONST = {tlm['nconst']};")
    c(f"  static constexpr int NSLOTS_TLM = {tlm['total']};")
    c("  // dy_new = d(y_new)/d(y, k) (dy, dk) for one step of size h: walks")
    c("  // coop::tlm_prog.  Requires attempt() for this step first (the LU of W and")
    c("  // the K_i), y_n in S[Y..], dy in S[DYT..] and dk in S[DKR..].")
    c("  template <class SA, class KA>")
    c("  __device__ __forceinline__ static void tlm_step(SA& S, const KA& k, double h) {")
    c("    for (int r = 0; r < NR; ++r) S[KT + r] = k(r);")
    c("    for (int i = 0; i < TLM_NCONST; ++i) S[TLM_CB + i] = coop::tlm_const_val[i];")
    for (st, j), slot in tlm["cterm"].items():
        cv = C[(st - 1) * (st - 2) // 2 + j - 1]
        c(f"    S[{slot}] = {_lit(cv)} / h;    // c{st}{j} / h")
    c("    for (int n = 0; n < coop::TLM_OPS; ++n) {")
    c("      const unsigned long long w = __ldg(coop::tlm_prog + n);")
    c("      const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);")
    c("      const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^")
    c("                                            ((long long)(lo >> 31) << 63));")
    c("      S[lo & 0xffffu] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);")
    c("    }")
    c("  }")


def _emit_table_adjoint(c, coop):
    """Table-driven adjoint_step: one thread walks the reverse-step program
    (``_adjoint_program``) on its own cell."""
    adj = coop["adj"]
    c("")
    c("  // ---- discrete adjoint of one accepted step (table-driven) ----")
    c(f"  static constexpr int LAM = {adj['LAM']};      // dL/dy")
    c(f"  static constexpr int KBAR = {adj['KBAR']};    // stage adjoints, NSTAGE x NV")
    c(f"  static constexpr int FBAR = {adj['FBAR']};    // adjoint of the pending stage tendency")
    c(f"  static constexpr int KB = {adj['KB']};        // dL/dk accumulated")
    c("  static constexpr int NSLOTS_ADJ = NSLOTS;")
    c("  // Reverse of one accepted step of size h: walks coop::adj_prog, the")
    c("  // arithmetic of the unrolled adjoint step operation by operation.")
    c("  // Requires attempt() for this step first (LU, K_i, and the constants and")
    c("  // rate constants it writes for h), y_n in S[Y..] and lambda in S[LAM..].")
    c("  template <class SA, class KA>")
    c("  __device__ __forceinline__ static void adjoint_step(SA& S, const KA& k, double h) {")
    c("    (void)k;")
    c("    (void)h;")
    c("    for (int n = 0; n < coop::ADJ_OPS; ++n) {")
    c("      const unsigned long long w = __ldg(coop::adj_prog + n);")
    c("      const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);")
    c("      const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^")
    c("                                            ((long long)(lo >> 31) << 63));")
    c("      S[lo & 0xffffu] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);")
    c("    }")
    c("  }")
    c("")
    c("  // ---- tendencies and Jacobian (table-driven evaluation entries) ----")
    c("  // For y in S[Y..]: F(y) into S[F..] and W with 1/(gamma h) = 0, that is")
    c("  // -J, into the W slots of the LU store.  Walks coop::eval_prog, the")
    c("  // first stage's partials, W and F code without the factorization.")
    c("  template <class SA, class KA>")
    c("  __device__ __forceinline__ static void eval_step(SA& S, const KA& k) {")
    c("    for (int r = 0; r < NR; ++r) S[KT + r] = k(r);")
    c("    for (int i = 0; i < NCONST; ++i) S[CB + i] = coop::const_val[i];")
    c("    S[CB + 3] = 0.0;  // 1/(gamma h)")
    c("    for (int n = 0; n < coop::EVAL_OPS; ++n) {")
    c("      const unsigned long long w = __ldg(coop::eval_prog + n);")
    c("      const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);")
    c("      const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^")
    c("                                            ((long long)(lo >> 31) << 63));")
    c("      S[lo & 0xffffu] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);")
    c("    }")
    c("  }")


def _emit_table_attempt_head(c, coop, C):
    """Head of the table-driven per-thread attempt (the increment and error
    norm that follow are those of the unrolled attempt)."""
    c("  // One Rosenbrock attempt of size h from the state in S[Y..], table-driven:")
    c("  // one thread walks the stage programs of the cooperative kernel")
    c("  // (coop::sched) on its own cell, step after step, the words of a step in")
    c("  // order.  The operations of a step are independent, so the order changes")
    c("  // no bit, and all lanes of a warp read the same word.  Returns the WRMS")
    c("  // error norm and leaves the increment sum_j M_j K_j in S[DY..]; bit 1 of")
    c("  // status is set on a zero pivot.")
    c("  template <class SA, class KA>")
    c("  __device__ __forceinline__ static double attempt(SA& S, const KA& k, double h, int& status) {")
    c("    for (int r = 0; r < NR; ++r) S[KT + r] = k(r);")
    c("    for (int i = 0; i < NCONST; ++i) S[CB + i] = coop::const_val[i];")
    c("    S[CB + 3] = 1.0 / (GAMMA * h);")
    for (st, j), slot in coop["cterm_slot"].items():
        cv = C[(st - 1) * (st - 2) // 2 + j - 1]
        c(f"    S[{slot}] = {_lit(cv)} / h;    // c{st}{j} / h")
    c("    bool ok = true;")
    c("    const int steps = coop::stage_step[NSTAGE];")
    c("    for (int s = 0; s < steps; ++s) {")
    c("      const unsigned long long* __restrict__ row = coop::sched + (size_t)s * 32;")
    c("      for (int j = 0; j < 32; ++j) {")
    c("        const unsigned long long w = __ldg(row + j);")
    c("        const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);")
    c("        const unsigned out = lo & 0xffffu;")
    c("        if (out == 0xffffu) break;          // a step's idle lanes come last")
    c("        if (hi >> 31) {")
    c("          const double v = S[out];")
    c("          ok = ok && (v != 0.0);")
    c("          S[out] = 1.0 / v;")
    c("        } else {")
    c("          const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^")
    c("                                                ((long long)(lo >> 31) << 63));")
    c("          S[out] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);")
    c("        }")
    c("      }")
    c("    }")
    c("    if (!ok) status |= 1;")


def _emit_coop(c, plan, coop, nv, ns, stages, C, M, E, K0, Y, FS, DY):
    """Warp-cooperative form of one attempt: the stage programs of
    ``_coop_build`` run as static 32-lane schedules.  Used for the few cells
    whose step count makes one lane too slow, and (``table`` mechanisms) as
    the table that the per-thread interpreter walks."""
    progs, sched, npart, nq = coop["progs"], coop["sched"], coop["npart"], coop["nq"]
    Q, D, CB, nconst = coop["Q"], coop["D"], coop["CB"], coop["nconst"]
    const_vals, literals, cterm_slot, Mech_KT = coop["const_vals"], coop["literals"], coop["cterm_slot"], coop["KT"]
    c("")
    c("  // ---- warp-cooperative attempt (static warp schedules) ----")
    c(f"  static constexpr int NPART = {npart};")
    c(f"  static constexpr int Q = {Q};            // rates q_r, then q_i of the error norm")
    c(f"  static constexpr int D = {D};     // partial derivatives")
    c(f"  static constexpr int CB = {CB};        // constants")
    c(f"  static constexpr int NCONST = {nconst};")
    c(f"  static constexpr int COOP_SLOTS = CB + NCONST;")
    t = _Code()
    t("// Tables of the warp-cooperative attempt (device constant data).")
    t("namespace coop {")
    t(f"static __device__ const double const_val[{nconst}] = {{{', '.join(const_vals)}}};")
    offs = [0]
    for st_ in sched:
        offs.append(offs[-1] + len(st_))
    t(f"static __device__ const int stage_step[{len(offs)}] = {{{', '.join(map(str, offs))}}};")
    words = []
    for ops, st_ in zip(progs, sched):
        words += warp_schedule.encode(ops, st_)
    _c_u64_array(t, "sched", words)
    if coop["adj_ops"] is not None:
        ops = coop["adj_ops"]
        t(f"constexpr int ADJ_OPS = {len(ops)};")
        _c_u64_array(t, "adj_prog", warp_schedule.encode(ops, [[i] for i in range(len(ops))], lanes=1))
    if coop["eval_ops"] is not None:
        ops = coop["eval_ops"]
        t(f"constexpr int EVAL_OPS = {len(ops)};")
        _c_u64_array(t, "eval_prog", warp_schedule.encode(ops, [[i] for i in range(len(ops))], lanes=1))
    tlm = _tlm_build(plan, nv, stages, coop["A"], C, M, coop["NewF"], K0, Y, Mech_KT, coop["total"])
    tlm_code = _Code()
    _emit_tlm(tlm_code, t, tlm, C)
    plan._tlm = tlm
    t("}  // namespace coop")
    t("")
    plan._coop_tables = t.text()
    plan._coop_programs = (progs, sched, {"CB": CB, "nconst": nconst, "literals": dict(literals),
                                          "cterm_slot": dict(cterm_slot), "Y": Y, "K0": K0, "FS": FS,
                                          "DY": DY, "KT": Mech_KT, "C": list(C), "slots": CB + nconst})
    c("  // Run steps [s_begin, s_end) of the static warp schedule on S: one")
    c("  // uniform operation S[out] = fma(+-S[a], S[b], S[c]) (or a pivot")
    c("  // reciprocal) per lane and step, a warp barrier between steps.  The words")
    c("  // of the next SCHED_AHEAD steps are in flight while the current ones")
    c("  // execute; words past the end read as idle lanes.  Returns false if a")
    c("  // reciprocal met a zero pivot.")
    c("  static constexpr int SCHED_AHEAD = 8;")
    c("  __device__ __forceinline__ static bool run_schedule(double* S, int s_begin, int s_end, unsigned lane) {")
    c("    const unsigned long long* __restrict__ T = coop::sched;")
    c("    bool ok = true;")
    c("    unsigned long long cur[SCHED_AHEAD];")
    c("    #pragma unroll")
    c("    for (int j = 0; j < SCHED_AHEAD; ++j) {")
    c("      const int s = s_begin + j;")
    c("      cur[j] = s < s_end ? __ldg(T + (size_t)s * 32 + lane) : 0xffffull;")
    c("    }")
    c("    for (int s0 = s_begin; s0 < s_end; s0 += SCHED_AHEAD) {")
    c("      unsigned long long nxt[SCHED_AHEAD];")
    c("      #pragma unroll")
    c("      for (int j = 0; j < SCHED_AHEAD; ++j) {")
    c("        const int s = s0 + SCHED_AHEAD + j;")
    c("        nxt[j] = s < s_end ? __ldg(T + (size_t)s * 32 + lane) : 0xffffull;")
    c("      }")
    c("      #pragma unroll")
    c("      for (int j = 0; j < SCHED_AHEAD; ++j) {")
    c("        const unsigned long long w = cur[j];")
    c("        const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);")
    c("        const unsigned out = lo & 0xffffu;")
    c("        if (out != 0xffffu) {")
    c("          if (hi >> 31) {")
    c("            const double v = S[out];")
    c("            ok = ok && (v != 0.0);")
    c("            S[out] = 1.0 / v;")
    c("          } else {")
    c("            // Negation flips the sign bit: exact, like -x in the per-thread code.")
    c("            const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^")
    c("                                                  ((long long)(lo >> 31) << 63));")
    c("            S[out] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);")
    c("          }")
    c("        }")
    c("        __syncwarp();")
    c("      }")
    c("      #pragma unroll")
    c("      for (int j = 0; j < SCHED_AHEAD; ++j) cur[j] = nxt[j];")
    c("    }")
    c("    return ok;")
    c("  }")
    c("")
    c("  // One attempt by a whole warp on the cell held in shared memory S")
    c("  // (COOP_SLOTS doubles; the rate constants in the KT slots).  Same values")
    c("  // as attempt(); the error norm is summed by lane 0 in species order.")
    c("  // Returns err on every lane.")
    c("  template <class KA>")
    c("  __device__ __forceinline__ static double attempt_coop(double* S, const KA& k, double h, int& status,")
    c("                                                       unsigned lane) {")
    c("    (void)k;")
    c("    namespace T = coop;")
    c("    for (int i = lane; i < NCONST; i += 32) S[CB + i] = T::const_val[i];")
    c("    __syncwarp();")
    c("    if (lane == 0) {")
    c("      S[CB + 3] = 1.0 / (GAMMA * h);")
    for (st, j), slot in cterm_slot.items():
        cv = C[(st - 1) * (st - 2) // 2 + j - 1]
        c(f"      S[{slot}] = {_lit(cv)} / h;    // c{st}{j} / h")
    c("    }")
    c("    __syncwarp();")
    c("    bool ok = true;")
    c("    for (int st = 0; st < NSTAGE; ++st) ok = run_schedule(S, T::stage_step[st], T::stage_step[st + 1], lane) && ok;")
    c("    if (__any_sync(0xffffffffu, !ok)) status |= 1;")
    mterms = [(M[j], j) for j in range(stages) if M[j] != 0.0]
    eterms = [(E[j], j) for j in range(stages) if E[j] != 0.0]

    def lin(terms):
        expr = None
        for cv, j in terms:
            t_ = f"k{j}"
            if expr is None:
                expr = t_ if cv == 1.0 else f"{_lit(cv)} * {t_}"
            else:
                expr = f"{expr} + {t_}" if cv == 1.0 else f"fma({_lit(cv)}, {t_}, {expr})"
        return expr or "0.0"
    c("    // Increment, and q_i^2 of the error norm into the rate slots.")
    c("    for (int i = lane; i < NV; i += 32) {")
    for j in range(stages):
        c(f"      const double k{j} = S[{K0 + j * nv} + i];")
    c("      const double yi = S[Y + i];")
    ynew = "yi"
    for cv, j in mterms:
        ynew = f"{ynew} + k{j}" if cv == 1.0 else f"fma({_lit(cv)}, k{j}, {ynew})"
    c(f"      const double ynew = {ynew};")
    c(f"      S[DY + i] = {lin(mterms)};")
    c("      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));")
    c(f"      S[Q + i] = ({lin(eterms)}) / sc;")
    c("    }")
    c("    __syncwarp();")
    c("    double err = 0.0;")
    c("    if (lane == 0) {")
    c("      double err_sq = 0.0;")
    c("      for (int i = 0; i < NV; ++i) err_sq = fma(S[Q + i], S[Q + i], err_sq);")
    c(f"      err = fmax(sqrt(err_sq / {ns}.0), 1.0e-10);")
    c("    }")
    c("    return __shfl_sync(0xffffffffu, err, 0);")
    c("  }")
    for line in tlm_code.lines:
        c(line)


def _monomial_terms(reactants, v2l):
    """Exponents {logical species: power} of a reaction's variable monomial."""
    m = {}
    for s_, pw in reactants:
        m[v2l[s_]] = m.get(v2l[s_], 0) + pw
    return m


def _mono_expr(expo, yname):
    """C expression of prod y^e (factors repeated), '1.0' if empty."""
    fac = []
    for j in sorted(expo):
        fac += [f"{yname}{j}"] * expo[j]
    return " * ".join(fac) if fac else "1.0"


def _dmono(expo, j):
    """(coefficient, exponents) of d/dy_j of prod y^e, or None."""
    if expo.get(j, 0) == 0:
        return None
    e = dict(expo)
    c = e[j]
    e[j] -= 1
    if e[j] == 0:
        del e[j]
    return float(c), e


def _emit_adjoint(c, plan, nv, nr, stages, A, C, M, NewF, K0, Y, nslots):
    """Discrete adjoint of one accepted step (reverse of ``attempt``).

    Given lambda = dL/dy_{n+1} in S[LAM..] and the stage values of the step
    recomputed by ``attempt`` (LU of W, K_i, y_n), overwrite S[LAM..] with
    dL/dy_n and add dL/dk to S[KB..].  W = I/(gamma h) - J(y_n, k) and
    f = sum_r net_r k_r m_r(y) (mass action), so every derivative is a sum
    over reactions: (df/dk)^T Fbar, J^T Fbar, and the W terms
    u^T dJ v = sum_r k_r (net_r.u) (H_r v . dy + grad m_r . v dk_r/k_r).
    """
    v2l = plan.phys_to_var
    LAM = nslots
    KBAR = LAM + nv
    FBAR = KBAR + stages * nv
    KB = FBAR + nv
    nadj = KB + nr
    c("")
    c("  // ---- discrete adjoint of one accepted step ----")
    c(f"  static constexpr int LAM = {LAM};      // dL/dy")
    c(f"  static constexpr int KBAR = {KBAR};    // stage adjoints, NSTAGE x NV")
    c(f"  static constexpr int FBAR = {FBAR};    // adjoint of the pending stage tendency")
    c(f"  static constexpr int KB = {KB};        // dL/dk accumulated")
    c(f"  static constexpr int NSLOTS_ADJ = {nadj};")
    # With the adjoint state in the global tile (more slots than the register
    # store holds), the two largest adjoint-only helpers are compiled once as
    # out-of-line functions instead of once per stage: this bounds the size
    # of the adjoint kernel's body, which sets its compile time.  Register
    # stores stay inlined, since a call would move them to local memory.
    adj_inline = "__noinline__" if nadj > REGISTER_SLOTS else "__forceinline__"
    # transposed solve: W^T x = b  with W = LU: U^T z = b (forward), L^T x = z (backward)
    ucol = [[] for _ in range(nv)]   # U(k, i), k < i
    lcol = [[] for _ in range(nv)]   # L(k, i), k > i
    for (r_, cc), sl in plan.lu_index.items():
        if r_ < cc:
            ucol[cc].append((r_, sl))
        elif r_ > cc:
            lcol[cc].append((r_, sl))
    c("  // Solve W^T x = b in place on [base, base + NV) with the stored LU of W.")
    c("  template <class SA>")
    c(f"  __device__ {adj_inline} static void solve_t(SA& S, const int base) {{")
    for i in range(nv):
        expr = f"S[base + {i}]"
        for k_, sl in sorted(ucol[i]):
            expr = f"fma(-S[{sl}], z{k_}, {expr})"
        c(f"    const double z{i} = ({expr}) * S[{plan.diag[i]}];")
    for i in range(nv - 1, -1, -1):
        expr = f"z{i}"
        for k_, sl in sorted(lcol[i]):
            expr = f"fma(-S[{sl}], x{k_}, {expr})"
        c(f"    const double x{i} = {expr};")
        c(f"    S[base + {i}] = x{i};")
    c("  }")
    c("")
    # per-reaction helpers
    rx = []
    for r in plan.reactions:
        expo = _monomial_terms(r.reactants, v2l)
        net = [(v2l[s_], co) for s_, co in r.net]
        rx.append((r.index, expo, net))

    def dot_net(net, uname):
        terms = [(co, f"{uname}({i})") for i, co in net]
        return _sum_expr(None, terms)

    # W term: u^T dJ(y) v  -> dy and dk contributions
    c("  // u^T J(y) v terms of stage i: y in S[Y..], u in S[ub..], v = K_i in S[vb..].")
    c("  template <class SA, class KA>")
    c(f"  __device__ {adj_inline} static void adj_wterm(SA& S, const KA& k, const int ub, const int vb) {{")
    c("    auto u = [&](int i) { return S[ub + i]; };")
    used = sorted({j for _, e, _ in rx for j in e})
    for j in used:
        c(f"    const double y{j} = S[Y + {j}];")
        c(f"    const double v{j} = S[vb + {j}];")
    acc_y = {}
    for ri, expo, net in rx:
        if not net or not expo:
            continue
        c(f"    {{ const double s = {dot_net(net, 'u')};")
        # grad m . v
        gterms = []
        for j in sorted(expo):
            d = _dmono(expo, j)
            coef, e2 = d
            gterms.append((coef, f"({_mono_expr(e2, 'y')}) * v{j}" if e2 else f"v{j}"))
        c(f"      S[KB + {ri}] = fma(s, {_sum_expr(None, gterms)}, S[KB + {ri}]);")
        c(f"      const double ks = k({ri}) * s;")
        # H v: for each p: sum_q d2m/dy_p dy_q v_q
        for p_ in sorted(expo):
            d1 = _dmono(expo, p_)
            hterms = []
            for q in sorted(d1[1]):
                d2 = _dmono(d1[1], q)
                coef = d1[0] * d2[0]
                hterms.append((coef, f"({_mono_expr(d2[1], 'y')}) * v{q}" if d2[1] else f"v{q}"))
            if hterms:
                c(f"      S[LAM + {p_}] = fma(ks, {_sum_expr(None, hterms)}, S[LAM + {p_}]);")
        c("    }")
    c("  }")
    c("")
    # F term at a stage state Y_i given Fbar: J(Y)^T Fbar into LAM and (df/dk)^T Fbar into KB,
    # and the Y-adjoint returned through out(j, value) for the K_j contributions.
    c("  // Adjoint of F_i = f(Y_i): Ybar = J(Y_i)^T Fbar, kbar += m_r(Y_i) (net_r.Fbar).")
    c("  // yv(i) supplies Y_i, ybar(j, x) receives Ybar_j.")
    c("  template <class SA, class KA, class YA, class OUT>")
    c("  __device__ __forceinline__ static void adj_fterm(SA& S, const KA& k, const YA& yv, OUT&& ybar) {")
    c("    auto fb = [&](int i) { return S[FBAR + i]; };")
    for j in used:
        c(f"    const double y{j} = yv({j});")
    yb_terms = {j: [] for j in range(nv)}
    for ri, expo, net in rx:
        if not net:
            continue
        c(f"    const double s{ri} = {dot_net(net, 'fb')};")
        c(f"    S[KB + {ri}] = fma(s{ri}, {_mono_expr(expo, 'y')}, S[KB + {ri}]);")
        for j in sorted(expo):
            coef, e2 = _dmono(expo, j)
            mono = _mono_expr(e2, 'y')
            t = f"k({ri}) * s{ri}" + ("" if mono == "1.0" else f" * {mono}")
            yb_terms[j].append((coef, t))
    for j in range(nv):
        if yb_terms[j]:
            c(f"    ybar({j}, {_sum_expr(None, yb_terms[j])});")
    c("  }")
    c("")
    # adjoint step
    c("  // Reverse of one accepted step of size h.  Requires the values attempt()")
    c("  // left in S for this step (LU, K_i) and y_n in S[Y..].")
    c("  template <class SA, class KA>")
    c("  __device__ __forceinline__ static void adjoint_step(SA& S, const KA& k, double h) {")
    for i in range(stages):
        mi = M[i]
        c("    #pragma unroll")
        c("    for (int j = 0; j < NV; ++j) S[KBAR + " + str(i * nv) + " + j] = "
          + (f"{_lit(mi)} * S[LAM + j];" if mi != 0.0 else "0.0;"))
    c("    #pragma unroll")
    c("    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;")
    # src stage for each stage's F
    src = []
    last = 0
    for i in range(stages):
        if NewF[i]:
            last = i
        src.append(last)
    for i in range(stages - 1, -1, -1):
        kb_i = f"KBAR + {i * nv}"
        c(f"    // stage {i + 1}")
        c(f"    solve_t(S, {kb_i});                       // u_i = W^-T Kbar_i")
        c(f"    adj_wterm(S, k, {kb_i}, {K0 + i * nv});       // J(y_n) in W")
        c("    #pragma unroll")
        c(f"    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[{kb_i} + j];")
        for j in range(i):
            cv = C[i * (i - 1) // 2 + j]
            if cv != 0.0:
                c(f"    {{ const double cc = {_lit(cv)} / h;")
                c("      #pragma unroll")
                c(f"      for (int q = 0; q < NV; ++q) S[KBAR + {j * nv} + q] = fma(cc, S[{kb_i} + q], S[KBAR + {j * nv} + q]); }}")
        if NewF[i]:
            # Y_i = y_n + sum_j a_ij K_j
            aterms = [(A[i * (i - 1) // 2 + j], j) for j in range(i) if i > 0 and A[i * (i - 1) // 2 + j] != 0.0]
            yexpr = "S[Y + q]"
            for a, j in aterms:
                kk = f"S[{K0 + j * nv} + q]"
                yexpr = f"{yexpr} + {kk}" if a == 1.0 else f"{yexpr} + {_lit(a)} * {kk}"
            acc_lines = ["S[LAM + j] += x;"]
            for a, j in aterms:
                acc_lines.append(f"S[KBAR + {j * nv} + j] = fma({_lit(a)}, x, S[KBAR + {j * nv} + j]);")
            c(f"    adj_fterm(S, k, [&](int q) {{ return {yexpr}; }},")
            c(f"              [&](int j, double x) {{ {' '.join(acc_lines)} }});")
            c("    #pragma unroll")
            c("    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;")
    c("  }")


# Above this many LU multiply-adds the per-thread attempt is table-driven
# (TS1: 49299) instead of unrolled (SAPRC99: 9654, which already costs one to
# two minutes of cicc + ptxas per kernel).
TABLE_PRODUCTS = 20000


def emit_mechanism(plan: ReducedPlan, table: bool | None = None) -> str:
    """Device header of one mechanism.  `table`: per-thread attempt and
    adjoint step walking programs (the cooperative stage programs, the
    reverse-step program) instead of unrolled code (default: above
    TABLE_PRODUCTS LU multiply-adds)."""
    if table is None:
        table = len(plan.products) > TABLE_PRODUCTS
    raw = plan.raw
    name = plan.name
    nv, ns, nr = plan.n_var, plan.n_species, len(plan.reactions)
    v2l = plan.phys_to_var
    tab = plan.tableau
    stages = int(tab["stages"])
    A, C, M, E, NewF = tab["A"], tab["C"], tab["M"], tab["E"], tab["NewF"]
    gamma0 = tab["Gamma"][0]
    elo = float(tab["ELO"])
    nlu = len(plan.lu_slots)
    np_ = max(1, plan.num_rate_parameters)
    nfix = len(plan.fixed_phys)
    c = _Code()
    c(f"// Generated by mkpp_gb300.emitter.cuda_emitter from mechanisms/{name}.plan.json.")
    c("// Do not edit: regenerate with `python -m mkpp_gb300.emitter.cuda_emitter`.")
    c(f"// {ns} species ({nv} variable), {nr} reactions, {len(plan.w_slots)} W slots, "
      f"{nlu} LU slots, {plan.lu_fma} LU products, {plan.lu_div} pivot scalings.")
    c("#pragma once")
    c('#include "mkpp_device.cuh"')
    c(f"namespace mkpp_{name} {{")
    c("")
    c("struct Mech {")
    c(f'  static constexpr const char* NAME = "{name}";')
    c(f"  static constexpr int NS = {ns};      // species including fixed ones")
    c(f"  static constexpr int NV = {nv};      // variable species (solved system)")
    c(f"  static constexpr int NR = {nr};      // reactions")
    c(f"  static constexpr int NP = {plan.num_rate_parameters};      // runtime parameter slots per cell")
    c(f"  static constexpr int NPH = {plan.num_photolysis};      // photolysis slots")
    c(f"  static constexpr int NFIX = {nfix};")
    c(f"  static constexpr int NLU = {nlu};")
    c(f"  static constexpr int NSTAGE = {stages};")
    c(f"  static constexpr bool RUNTIME_ENV = {'true' if plan.runtime_environment else 'false'};")
    c(f"  static constexpr bool CLOUD_GATED = {'true' if plan.cloud_gated else 'false'};")
    c(f"  static constexpr double GAMMA = {_lit(gamma0)};")
    c(f"  static constexpr double ELO = {_lit(elo)};")
    c(f"  static constexpr double SEED = {_lit(plan.seed)};")
    c(f"  static constexpr double ENV_T = {_lit(raw['environment_temperature'])};")
    c(f"  static constexpr double ENV_RHO = {_lit(raw['environment_air_density'])};")
    c(f"  static constexpr long long LU_FMA = {plan.lu_fma};")
    c(f"  static constexpr long long LU_SCALE = {plan.lu_div};")
    low, up = plan.solve_entries
    c(f"  static constexpr long long SOLVE_L = {low};")
    c(f"  static constexpr long long SOLVE_U = {up};")
    # Algorithmic FP64 operations of F and of the Jacobian partials per
    # evaluation (a multiply-add counts two); plan.flops_per_attempt adds
    # the LU, solves, stages and error norm.
    fun_fl = sum(max(0, sum(pw for _, pw in r.reactants)) for r in plan.reactions) + \
        sum(2 * len(r.net) for r in plan.reactions)
    jac_fl = sum(2 * len(r.net) * len(r.reactants) for r in plan.reactions) + \
        sum(len(r.reactants) * max(0, sum(pw for _, pw in r.reactants) - 1) for r in plan.reactions)
    c(f"  static constexpr long long FUN_FLOPS = {fun_fl};")
    c(f"  static constexpr long long JAC_FLOPS = {jac_fl};")
    c("")
    # physical index tables
    c(f"  __host__ __device__ static constexpr int var_phys(int i) {{ constexpr int t[{nv}] = {{"
      + ", ".join(str(x) for x in plan.var_phys) + "}; return t[i]; }")
    if nfix:
        c(f"  __host__ __device__ static constexpr int fix_phys(int i) {{ constexpr int t[{nfix}] = {{"
          + ", ".join(str(x) for x in plan.fixed_phys) + "}; return t[i]; }")
    else:
        c("  __host__ __device__ static constexpr int fix_phys(int) { return 0; }")
    c(f"  __host__ __device__ static constexpr double atol_v(int i) {{ constexpr double t[{nv}] = {{"
      + ", ".join(_lit(plan.atol[p]) for p in plan.var_phys) + "}; return t[i]; }")
    c(f"  __host__ __device__ static constexpr double rtol_v(int i) {{ constexpr double t[{nv}] = {{"
      + ", ".join(_lit(plan.rtol[p]) for p in plan.var_phys) + "}; return t[i]; }")
    # Tolerances of every species in physical order, the reference's
    # SolverKernels::atol[] / rtol[] (host queries; the solve uses the above).
    c(f"  static constexpr double ATOL[NS] = {{" + ", ".join(_lit(x) for x in plan.atol) + "};")
    c(f"  static constexpr double RTOL[NS] = {{" + ", ".join(_lit(x) for x in plan.rtol) + "};")
    c(f"  __host__ __device__ static constexpr int lu_prow(int s) {{ constexpr int t[{nlu}] = {{"
      + ", ".join(str(plan.var_phys[r]) for r, _ in plan.lu_slots) + "}; return t[s]; }")
    c(f"  __host__ __device__ static constexpr int lu_pcol(int s) {{ constexpr int t[{nlu}] = {{"
      + ", ".join(str(plan.var_phys[cc]) for _, cc in plan.lu_slots) + "}; return t[s]; }")
    names = ", ".join('"%s"' % x for x in raw["species"])
    c(f"  static const char* species_name(int s) {{ static const char* t[{ns}] = {{{names}}}; return t[s]; }}")
    # The reference names photolysis slots J_1..J_n (mkpp_c_api.cpp.j2:33-38).
    if plan.num_photolysis:
        pnames = ", ".join('"J_%d"' % (i + 1) for i in range(plan.num_photolysis))
        c(f"  static const char* photolysis_name(int p) {{ static const char* t[{plan.num_photolysis}] = {{{pnames}}}; return t[p]; }}")
    else:
        c('  static const char* photolysis_name(int) { return ""; }')
    c("")
    # ---------------- rate constants
    c("  // Rate constants of every reaction (reaction index order).  P(n) is the")
    c("  // cell's runtime parameter n (photolysis J_n or external Rate slot n),")
    c("  // FIX(s) the concentration of fixed species s, T/RHO the cell's")
    c("  // temperature and air density.")
    c("  template <class PA, class FA, class KO>")
    c("  __device__ __forceinline__ static void rate_constants(const PA& P, const FA& FIX, double T, double RHO,")
    c("                                                      double RH, double CLW, KO& k) {")
    c("    (void)T; (void)RHO; (void)RH; (void)CLW; (void)P; (void)FIX;")
    for r in plan.reactions:
        c(f"    k.set({r.index}, {_k_text(r.k)});")
    c("  }")
    c("")
    # ---------------- storage layout
    nlu_ = nlu
    Y = nlu_
    K0 = Y + nv
    FS = K0 + stages * nv
    DY = FS + nv
    KT = DY + nv
    nslots = KT + nr
    c("  // Per-cell working storage, in slots of one double: the LU factors, the")
    c("  // state y, the stage vectors K_1..K_s, the tendency F, the increment dy and")
    c("  // the rate constants of the current host step.")
    c(f"  static constexpr int Y = {Y};")
    c(f"  static constexpr int K0 = {K0};")
    c(f"  static constexpr int F = {FS};")
    c(f"  static constexpr int DY = {DY};")
    c(f"  static constexpr int KT = {KT};        // the cell's rate constants for the current host step")
    coop = _coop_build(plan, nv, stages, A, C, NewF, K0, Y, FS, DY, nslots, table=table, M=M)
    if table:
        c("  // Table-driven attempt: the per-thread store holds all slots of the")
        c("  // stage programs (rates, partials, constants).")
        c(f"  static constexpr int NSLOTS = {coop['total']};")
    else:
        c(f"  static constexpr int NSLOTS = {nslots};")
    plan._nslots = coop["total"] if table else nslots
    c(f"  static constexpr bool TABLE_ATTEMPT = {'true' if table else 'false'};")
    c("")
    # With the store in the global tile, fun, jac_w, factor and solve are
    # compiled once each as out-of-line functions.  Inlined into the attempt,
    # the straight-line code of all four is one schedule in which loads are
    # hoisted far ahead of their use: for SAPRC99 the attempt then spilled a
    # 7.6 KB stack frame per thread (ncu, capped case: 42 GB of local-memory
    # traffic against 29 GB of tile traffic), and called out of line it
    # spills almost nothing and runs 29% more attempts per second.  Register
    # stores stay inlined, since a call would move them to local memory.
    store_slots = coop["total"] if table else nslots
    fn_inline = "__noinline__" if store_slots > REGISTER_SLOTS else "__forceinline__"
    # ---------------- Fun
    used_y_f = sorted({v2l[s_] for r in plan.reactions for s_, _ in r.reactants})
    c("  // Mass-action tendencies F(y) of the variable species (logical order):")
    c("  // y(i) supplies the state, out(i, F_i) receives the result.")
    c("  template <class YA, class KA, class FO>")
    c(f"  __device__ {fn_inline} static void fun(const YA& y, const KA& k, FO&& out) {{")
    for i in used_y_f:
        c(f"    const double y{i} = y({i});")
    rate_name = {}
    for r in plan.reactions:
        fac = [f"y{v2l[s_]}" for s_, pw in r.reactants for _ in range(pw)]
        term = " * ".join([f"k({r.index})"] + fac)
        c(f"    const double q{r.index} = {term};")
        rate_name[r.index] = f"q{r.index}"
    contrib = {i: [] for i in range(nv)}
    for r in plan.reactions:
        for s_, coef in r.net:
            contrib[v2l[s_]].append((coef, rate_name[r.index]))
    for i in range(nv):
        c(f"    out({i}, {_sum_expr(None, contrib[i])});")
    c("  }")
    c("")
    # ---------------- Jacobian -> W in LU slots
    c("  // W = I/(gamma h) - J(y) into the LU slots that hold W entries.")
    c("  template <class YA, class KA, class SA>")
    c(f"  __device__ {fn_inline} static void jac_w(const YA& y, const KA& k, double inv_g_dt, SA& S) {{")
    c("    (void)inv_g_dt;")
    used_y_j = sorted({v2l[s2] for r in plan.reactions if len(r.reactants) > 1 or any(pw > 1 for _, pw in r.reactants)
                       for s2, _ in r.reactants})
    for i in used_y_j:
        c(f"    const double y{i} = y({i});")
    partial_names = {}
    for r in plan.reactions:
        terms = list(r.reactants)
        for idx, (s_, pw) in enumerate(terms):
            others = []
            for jdx, (s2, pw2) in enumerate(terms):
                if jdx == idx:
                    if pw2 > 1:
                        others.append(_lit(float(pw2)))
                        others += [f"y{v2l[s2]}"] * (pw2 - 1)
                else:
                    others += [f"y{v2l[s2]}"] * pw2
            term = " * ".join([f"k({r.index})"] + others)
            nm = f"d{r.index}_{v2l[s_]}"
            partial_names[(r.index, s_)] = nm
            c(f"    const double {nm} = {term};")
    wterms = {loc: [] for loc in plan.w_slots}
    for r in plan.reactions:
        for s_, coef in r.net:
            for s2, _pw in r.reactants:
                wterms[(v2l[s_], v2l[s2])].append((-coef, partial_names[(r.index, s2)]))
    for loc in plan.w_slots:
        slot = plan.lu_index[loc]
        init = "inv_g_dt" if loc[0] == loc[1] else None
        c("    " + _accumulate(f"S[{slot}]", init, wterms[loc]))
    c("  }")
    c("")
    c("  // Physical (row, column) of every W slot, for the dense Jacobian.")
    c("  template <class Fn>")
    c("  __device__ __forceinline__ static void for_each_w_slot(Fn&& fn) {")
    for loc in plan.w_slots:
        c(f"    fn({plan.lu_index[loc]}, {plan.var_phys[loc[0]]}, {plan.var_phys[loc[1]]});")
    c("  }")
    c("")
    # ---------------- dense Jacobian: fixed-species columns
    c("  // Fixed-species columns of the dense Jacobian: dF_i/dC_f through the")
    c("  // rate constants' dependence on fixed species (third bodies).")
    c("  template <class PA, class FA, class YA, class Fn>")
    c("  __device__ __forceinline__ static void jac_fixed_columns(const PA& P, const FA& FIX, double T, double RHO,")
    c("                                                         double RH, double CLW, const YA& y, Fn&& fn) {")
    c("    (void)T; (void)RHO; (void)RH; (void)CLW; (void)P; (void)FIX; (void)y;")
    colterms: dict = {}
    for r, rr in zip(plan.reactions, raw["reactions"]):
        for fidx, dexpr in rr.get("dk_dfixed", []):
            mono = " * ".join(["(" + _k_text(dexpr) + ")"] + [f"y({v2l[s_]})" for s_, pw in r.reactants for _ in range(pw)])
            for s_, coef in r.net:
                colterms.setdefault((s_, fidx), []).append((coef, mono))
    for (row, col), terms in sorted(colterms.items()):
        c(f"    fn({row}, {col}, {_sum_expr(None, [(cf, '(' + t + ')') for cf, t in terms])});")
    c("  }")
    c("")
    # ---------------- LU factorization
    # (Table mode: the unrolled factor, solve and attempt are not emitted.)
    real_c = c
    if table:
        c = _Code()
    c("  // In-place row-wise Doolittle LU over the compact slots, in the operation")
    c("  // order of the reference plan.  The operands a row reuses (its own L")
    c("  // entries for the U part, the pivot column of U for the L part) are read")
    c("  // once into registers.  Diagonal slots end up holding 1/U_ii.")
    c("  template <class SA>")
    c(f"  __device__ {fn_inline} static bool factor(SA& S) {{")
    c("    bool ok = true;")
    diag_slots = set(plan.diag)
    slot_rc = plan.lu_slots
    # group ops by pivot row: U part (row == i) then L part (column == i)
    i_cur = None
    pre = {}
    def row_of(op):
        r, col = slot_rc[op[0]]
        return min(r, col)
    ops = plan.ops
    idx = 0
    while idx < len(ops):
        i = row_of(ops[idx])
        group = []
        while idx < len(ops) and row_of(ops[idx]) == i:
            group.append(ops[idx])
            idx += 1
        upart = [o for o in group if slot_rc[o[0]][0] == i]
        lpart = [o for o in group if slot_rc[o[0]][0] != i]
        c(f"    {{  // pivot row {i}")
        # preload the row's L entries used by the U part
        lslots = sorted({plan.products[q][0] for o in upart for q in range(o[2], o[3])})
        for sl in lslots:
            c(f"      const double a{sl} = S[{sl}];")
        # The diagonal U_ii comes first in the reference order; it only
        # depends on earlier rows, so it can be finished (and inverted) before
        # the rest of the row.  The remaining independent dot products of the
        # row advance together, one product per op per round, so the FP64 pipe
        # sees several independent chains; each op keeps its own product order.
        diag_op = [o for o in upart if o[0] in diag_slots]
        rest_u = [o for o in upart if o[0] not in diag_slots]
        for out, w, b, e, dg in diag_op:
            expr = f"S[{out}]" if w >= 0 else "0.0"
            for q in range(b, e):
                l_, u_ = plan.products[q]
                expr = f"fma(-a{l_}, S[{u_}], {expr})"
            c(f"      const double u{out} = {expr};")
            c(f"      ok = ok && (u{out} != 0.0);")
            c(f"      const double rd = 1.0 / u{out};")
            c(f"      S[{out}] = rd;")
        _interleave(c, plan, rest_u, lambda q: (f"a{plan.products[q][0]}", f"S[{plan.products[q][1]}]"), None)
        uslots = sorted({plan.products[q][1] for o in lpart for q in range(o[2], o[3])})
        for sl in uslots:
            c(f"      const double b{sl} = S[{sl}];")
        _interleave(c, plan, lpart, lambda q: (f"S[{plan.products[q][0]}]", f"b{plan.products[q][1]}"), "rd")
        c("    }")
    c("    return ok;")
    c("  }")
    c("")
    # ---------------- Solve
    c("  // Solve (LU) x = b in place on slots [base, base + NV): unit-L forward")
    c("  // sweep, then the U backward sweep scaled by the stored 1/U_ii.")
    c("  template <class SA>")
    c(f"  __device__ {fn_inline} static void solve(SA& S, const int base) {{")
    for i in range(nv):
        expr = f"S[base + {i}]"
        for col, slot in plan.lower[i]:
            expr = f"fma(-S[{slot}], v{col}, {expr})"
        c(f"    const double v{i} = {expr};")
    for i in range(nv - 1, -1, -1):
        expr = f"v{i}"
        for col, slot in plan.upper[i]:
            expr = f"fma(-S[{slot}], x{col}, {expr})"
        c(f"    const double x{i} = ({expr}) * S[{plan.diag[i]}];")
        c(f"    S[base + {i}] = x{i};")
    c("  }")
    c("")
    # ---------------- Attempt
    c("  // One Rosenbrock attempt of size h from the state in S[Y..].  Returns the")
    c("  // WRMS error norm and leaves the increment sum_j M_j K_j in S[DY..].")
    c("  // Bit 1 of status is set on a zero pivot.")
    c("  template <class SA, class KA>")
    c("  __device__ __forceinline__ static double attempt(SA& S, const KA& k, double h, int& status) {")
    c("    const double inv_g_dt = 1.0 / (GAMMA * h);")
    c("    jac_w([&](int i) { return S[Y + i]; }, k, inv_g_dt, S);")
    c("    if (!factor(S)) status |= 1;")
    for st in range(1, stages + 1):
        kb = K0 + (st - 1) * nv
        if NewF[st - 1]:
            if st == 1:
                c("    fun([&](int i) { return S[Y + i]; }, k, [&](int i, double v) { S[F + i] = v; });")
            else:
                terms = []
                for j in range(1, st):
                    a = A[(st - 1) * (st - 2) // 2 + j - 1]
                    if a != 0.0:
                        terms.append((a, j))
                expr = "S[Y + i]"
                for a, j in terms:
                    kk = f"S[{K0 + (j - 1) * nv} + i]"
                    expr = f"{expr} + {kk}" if a == 1.0 else f"{expr} + {_lit(a)} * {kk}"
                c(f"    fun([&](int i) {{ return {expr}; }}, k, [&](int i, double v) {{ S[F + i] = v; }});")
        cterms = []
        if st > 1:
            for j in range(1, st):
                cv = C[(st - 1) * (st - 2) // 2 + j - 1]
                if cv != 0.0:
                    cterms.append((cv, j))
        for cv, j in cterms:
            c(f"    const double c{st}{j} = {_lit(cv)} / h;")
        c("    #pragma unroll")
        c("    for (int i = 0; i < NV; ++i) {")
        expr = "S[F + i]"
        for cv, j in cterms:
            expr = f"fma(c{st}{j}, S[{K0 + (j - 1) * nv} + i], {expr})"
        c(f"      S[{kb} + i] = {expr};")
        c("    }")
        c(f"    solve(S, {kb});")
    if table:
        c = real_c
        _emit_table_attempt_head(c, coop, C)
    c("    double err_sq = 0.0;")
    c("    #pragma unroll")
    c("    for (int i = 0; i < NV; ++i) {")
    for j in range(stages):
        c(f"      const double k{j} = S[{K0 + j * nv} + i];")
    mterms = [(M[j], j) for j in range(stages) if M[j] != 0.0]
    eterms = [(E[j], j) for j in range(stages) if E[j] != 0.0]

    def lin(terms):
        expr = None
        for cv, j in terms:
            t = f"k{j}"
            if expr is None:
                expr = t if cv == 1.0 else f"{_lit(cv)} * {t}"
            else:
                expr = f"{expr} + {t}" if cv == 1.0 else f"fma({_lit(cv)}, {t}, {expr})"
        return expr or "0.0"

    # Ynew = ((S + K1) + M2 K2) + ... (integrate.j2 error block); the accepted
    # increment is K1 + M2 K2 + ... (integrate.j2 accept block).
    c("      const double yi = S[Y + i];")
    ynew = "yi"
    for cv, j in mterms:
        ynew = f"{ynew} + k{j}" if cv == 1.0 else f"fma({_lit(cv)}, k{j}, {ynew})"
    c(f"      const double ynew = {ynew};")
    c(f"      S[DY + i] = {lin(mterms)};")
    c("      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));")
    c(f"      const double q = ({lin(eterms)}) / sc;")
    c("      err_sq = fma(q, q, err_sq);")
    c("    }")
    c(f"    return fmax(sqrt(err_sq / {ns}.0), 1.0e-10);")
    c("  }")
    c("")
    c("  // Step-size factor from the error norm (integrate.j2:324-333).")
    c("  __device__ __forceinline__ static double growth(double err) {")
    if elo == 2.0:
        c("    const double fac = 0.9 / sqrt(err);")
    elif elo == 3.0:
        c("    const double fac = 0.9 / cbrt(err);")
    else:
        c(f"    const double fac = 0.9 * pow(err, -{_lit(1.0 / elo)});")
    c("    return fmax(0.2, fmin(fac, 6.0));")
    c("  }")
    _emit_coop(c, plan, coop, nv, ns, stages, C, M, E, K0, Y, FS, DY)
    if table:
        _emit_table_adjoint(c, coop)
    else:
        _emit_adjoint(c, plan, nv, nr, stages, A, C, M, NewF, K0, Y, nslots)
    c("};")
    c("")
    c(f"}}  // namespace mkpp_{name}")
    text = c.text()
    return text.replace("struct Mech {", plan._coop_tables + "\nstruct Mech {", 1)


def emit_host_header(plan) -> str:
    """generated/host_api/<m>/mkpp.h: the C ABI (include/mkpp.h) plus the
    mechanism's sizes, the per-mechanism constants of the reference's
    generated header (src/mkpp/templates/host_api/mkpp.h.j2:29-33)."""
    raw = plan.raw
    guard = f"MKPP_GB300_{plan.name.upper()}_MKPP_H"
    if not hasattr(plan, "_nslots"):
        emit_mechanism(plan)
    # The allocation-free entry's static scratch: NSLOTS doubles for each of
    # MKPP_NOALLOC_MAX_CELLS cells when the store is the global tile (more
    # than REGISTER_SLOTS slots), one double when it lives in registers.
    noalloc = (f"(MKPP_NOALLOC_MAX_CELLS * {plan._nslots} * 8)" if plan._nslots > REGISTER_SLOTS else "8")
    return f"""/*
 * mkpp.h of the {plan.name} library (libmkpp_{plan.name}.so), generated from its plan.
 * The C ABI of include/mkpp.h plus the mechanism's sizes, as the header the
 * reference generates per mechanism defines them
 * (src/mkpp/templates/host_api/mkpp.h.j2:29-33).  A host model built against
 * that header puts this directory on its include path instead.
 */
#ifndef {guard}
#define {guard}

#include "../../../../include/mkpp.h"

#define MKPP_NUM_RATE_PARAMETERS {raw["num_rate_parameters"]}
#define MKPP_NUM_SPECIES   {len(raw["species"])}
#define MKPP_NUM_REACTIONS {raw["num_reactions"]}
#define MKPP_NUM_PHOTOLYSIS {raw["num_photolysis"]}

/* Bytes of device memory that mkpp_gpu_integrate_noalloc's static scratch
 * holds on every GPU that loads this library, until the process exits. */
#define MKPP_NOALLOC_SCRATCH_BYTES {noalloc}

#endif
"""


def emit_solver_kernels_header(plan) -> str:
    """generated/host_api/<m>/<m>.hpp: the reference's generated C++ API of
    one mechanism (src/mkpp/templates/header.j2:70-80,127-203): namespace
    mkpp::generated::<m> with enum Species and SolverKernels<DeviceType>,
    here include/mkpp_gb300/solver_kernels.hpp bound to libmkpp_<m>.so."""
    raw = plan.raw
    name = plan.name
    ns = len(raw["species"])

    def lits(xs):
        return ", ".join(repr(float(x)) for x in xs)

    species = ",\n".join(f"    {sp} = {i}" for i, sp in enumerate(raw["species"]))
    pattern = ", ".join(f"{{{i}, {j}}}" for i, j in raw["jacobian_entries"])
    flag = lambda b: "true" if b else "false"  # noqa: E731
    return f"""// {name}.hpp of the {name} library (libmkpp_{name}.so), generated from its
// plan: the reference's generated C++ solver API for this mechanism
// (src/mkpp/templates/header.j2:70-80,127-203), namespace
// mkpp::generated::{name} with enum Species and SolverKernels<DeviceType>.
// The members and their execution are described in
// include/mkpp_gb300/solver_kernels.hpp.
#pragma once

#include "../../../../include/mkpp_gb300/solver_kernels.hpp"

namespace mkpp {{
namespace generated {{
namespace {name} {{

enum Species : int {{
{species}
}};

struct MechanismConstants {{
  static constexpr const char* NAME = "{name}";
  static constexpr int NUM_SPECIES = {ns};
  static constexpr int NUM_RUNTIME_PARAMETERS = {raw["num_rate_parameters"]};
  static constexpr int NUM_PHOTOLYSIS = {raw["num_photolysis"]};
  static constexpr int NUM_REACTIONS = {raw["num_reactions"]};
  static constexpr bool SUPPORTS_RUNTIME_ENVIRONMENT = {flag(raw["runtime_environment"])};
  static constexpr bool HAS_CLOUD_GATED = {flag(raw["cloud_gated"])};
  static constexpr double ENV_TEMPERATURE = {float(raw["environment_temperature"])!r};
  static constexpr double ENV_AIR_DENSITY = {float(raw["environment_air_density"])!r};
  static constexpr double INITIAL_STEP_SEED = {float(raw["initial_step_seed"])!r};
  static constexpr double atol[NUM_SPECIES] = {{{lits(raw["atol"])}}};
  static constexpr double rtol[NUM_SPECIES] = {{{lits(raw["rtol"])}}};
  // (row, column) of the Jacobian entries compute_jacobian writes
  static constexpr int NUM_JACOBIAN_ENTRIES = {len(raw["jacobian_entries"])};
  static constexpr int jacobian_pattern[NUM_JACOBIAN_ENTRIES][2] = {{{pattern}}};
}};

template <class DeviceType>
struct SolverKernels : ::mkpp_gb300::SolverKernelsBase<MechanismConstants, DeviceType> {{}};

}}  // namespace {name}
}}  // namespace generated
}}  // namespace mkpp
"""


def _write_if_changed(path: Path, text: str) -> None:
    path.parent.mkdir(parents=True, exist_ok=True)
    if not path.exists() or path.read_text() != text:
        path.write_text(text)


def write(name: str, out_dir: Path = GEN_DIR) -> Path:
    plan = load(name)
    path = out_dir / f"{name}.cuh"
    _write_if_changed(path, emit_mechanism(plan))
    _write_if_changed(out_dir / "host_api" / name / "mkpp.h", emit_host_header(plan))
    _write_if_changed(out_dir / "host_api" / name / f"{name}.hpp", emit_solver_kernels_header(plan))
    return path


def main(argv=None) -> int:
    import argparse

    ap = argparse.ArgumentParser(description="Emit sm_103a device headers from plan JSON")
    ap.add_argument("mechanisms", nargs="*", default=["chapman", "small_strato", "saprc99"])
    args = ap.parse_args(argv)
    for m in args.mechanisms:
        p = write(m)
        print(f"{m} -> {p} ({p.stat().st_size // 1024} KiB)")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())

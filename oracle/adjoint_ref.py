"""Dense FP64 CPU discrete adjoint (TEST INFRASTRUCTURE ONLY).

An independent NumPy restatement, on dense matrices, of the Rosenbrock step
of ``src/mkpp/templates/solver_variants/integrate.j2:144-263`` (W = I/(gamma h)
- J, K_i = W^-1 (F_i + sum_j C_ij/h K_j), Y_i = y + sum_j A_ij K_j,
y_new = y + sum_i M_i K_i) on the variable-species system, and of its
discrete adjoint for a given sequence of accepted step sizes.  The mass-action
tendency is f(y) = S (k * m(y)) with S the net stoichiometry and m_r the
reactant monomials, so J = S diag(k) Dm(y) and every second derivative is a
per-reaction monomial Hessian.  Used to check the GPU adjoint kernel.
"""

from __future__ import annotations

import numpy as np

from mkpp_gb300.emitter.plan import load


class DenseModel:
    def __init__(self, mechanism: str):
        p = load(mechanism)
        self.p = p
        nv, nr = p.n_var, len(p.reactions)
        self.nv, self.nr = nv, nr
        self.S = np.zeros((nv, nr))
        self.expo = []
        for r in p.reactions:
            for s, c in r.net:
                self.S[p.phys_to_var[s], r.index] += c
            e = {}
            for s, pw in r.reactants:
                e[p.phys_to_var[s]] = e.get(p.phys_to_var[s], 0) + pw
            self.expo.append(e)
        t = p.tableau
        self.st = int(t["stages"])
        self.A, self.C, self.M, self.NewF = t["A"], t["C"], t["M"], t["NewF"]
        self.g = t["Gamma"][0]

    def m(self, y):
        out = np.ones(self.nr)
        for r, e in enumerate(self.expo):
            for j, pw in e.items():
                out[r] *= y[j] ** pw
        return out

    def Dm(self, y):
        D = np.zeros((self.nr, self.nv))
        for r, e in enumerate(self.expo):
            for j, pw in e.items():
                v = float(pw) * y[j] ** (pw - 1)
                for j2, pw2 in e.items():
                    if j2 != j:
                        v *= y[j2] ** pw2
                D[r, j] = v
        return D

    def Hv(self, y, r, v):
        """Hessian of m_r at y times v."""
        e = self.expo[r]
        out = np.zeros(self.nv)
        for p_, pp in e.items():
            for q, pq in e.items():
                if p_ == q:
                    if pp < 2:
                        continue
                    val = pp * (pp - 1) * y[p_] ** (pp - 2)
                    for j2, pw2 in e.items():
                        if j2 != p_:
                            val *= y[j2] ** pw2
                else:
                    val = pp * y[p_] ** (pp - 1) * pq * y[q] ** (pq - 1)
                    for j2, pw2 in e.items():
                        if j2 not in (p_, q):
                            val *= y[j2] ** pw2
                out[p_] += val * v[q]
        return out

    def f(self, y, k):
        return self.S @ (k * self.m(y))

    def J(self, y, k):
        return self.S @ (k[:, None] * self.Dm(y))

    def a(self, i, j):
        return self.A[i * (i - 1) // 2 + j]

    def c(self, i, j):
        return self.C[i * (i - 1) // 2 + j]

    def step(self, y, k, h):
        W = np.eye(self.nv) / (self.g * h) - self.J(y, k)
        K, Ys, F = [], [], None
        for i in range(self.st):
            Yi = y + sum(self.a(i, j) * K[j] for j in range(i)) if i else y.copy()
            Ys.append(Yi)
            if self.NewF[i]:
                F = self.f(Yi, k)
            rhs = F + sum(self.c(i, j) / h * K[j] for j in range(i))
            K.append(np.linalg.solve(W, rhs))
        y_new = y + sum(self.M[i] * K[i] for i in range(self.st))
        return y_new, (W, K, Ys)

    def forward(self, y0, k, hs):
        y = y0.copy()
        tape = []
        for h in hs:
            y_new, stage = self.step(y, k, h)
            tape.append((y, h, stage))
            y = y_new
        return y, tape

    def adjoint(self, k, tape, lam):
        lam = lam.copy()
        kbar = np.zeros(self.nr)
        for y, h, (W, K, Ys) in reversed(tape):
            Kb = [self.M[i] * lam for i in range(self.st)]
            ybar = lam.copy()
            Fb = np.zeros(self.nv)
            for i in range(self.st - 1, -1, -1):
                u = np.linalg.solve(W.T, Kb[i])
                # u^T J(y) K_i with J = S diag(k) Dm(y)
                s = self.S.T @ u
                g = self.Dm(y) @ K[i]
                kbar += s * g
                for r in range(self.nr):
                    if s[r] != 0.0:
                        ybar += k[r] * s[r] * self.Hv(y, r, K[i])
                Fb += u
                for j in range(i):
                    Kb[j] = Kb[j] + self.c(i, j) / h * u
                if self.NewF[i]:
                    Yi = Ys[i]
                    sf = self.S.T @ Fb
                    kbar += sf * self.m(Yi)
                    Yb = self.Dm(Yi).T @ (k * sf)
                    ybar += Yb
                    for j in range(i):
                        Kb[j] = Kb[j] + self.a(i, j) * Yb
                    Fb = np.zeros(self.nv)
            lam = ybar
        return lam, kbar

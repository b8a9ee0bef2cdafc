"""Static 32-lane schedules of the warp-cooperative Rosenbrock attempt.

The warp-cooperative attempt runs one cell on a whole warp, so that the few
cells that need thousands of attempts in one host step finish sooner than on
a single lane.  Each tableau stage of the attempt (the Jacobian partials, W,
the fill-in zeros, the LU factorisation, F, the right-hand side and the
triangular solve) is one *program*: the per-thread kernel's scalar floating
point operations, in its order, each written as one uniform operation on
the per-cell store S in shared memory:

    FMA  S[out] = fma(+-S[a], S[b], S[c])
    RCP  S[out] = 1 / S[out]          (a pivot; zero flags the matrix singular)

Constant slots holding 1, +0, -0, the mechanism's literal coefficients and
the attempt's 1/(gamma h) and c_ij/h make every other form exact:

    x * y           fma(x, y, -0)          round(x * y); x*y + (-0) keeps the sign of zero
    x (copy)        fma(x, 1, -0)
    -x              fma(-x, 1, -0)
    0.0             fma(+0, +0, +0)
    acc + t         fma(t, 1, acc)         round(t + acc)
    acc - t         fma(-t, 1, acc)
    fma(c, t, acc)  fma(c, t, acc)

So every slot receives exactly the roundings of the per-thread kernel (which
is built with --fmad=false, so only its explicit fma() calls fuse), and a
cell gives the same bits on either kernel.

Dependencies are the read-after-write, write-after-read and write-after-write
hazards on slots, in program order.  A list scheduler (longest remaining
dependency path first) packs the operations into steps of at most 32; the
device runs one step per warp barrier.  On SAPRC99 the LU alone keeps ~31
lanes busy; the solves, whose row sums keep a fixed order, allow ~2.7.

Encoding, one 64-bit word per lane and step:
  bits 0-15 out | 16-30 a | 31 negate a | 32-47 b | 48-62 c | 63 reciprocal.
An idle lane holds out = 0xffff.
"""

from __future__ import annotations

import heapq

FMA, RCP = 1, 2
LANES = 32
IDLE = 0xFFFF


class Program:
    """Sequential uniform operations, built in per-thread program order.

    `zn`, `zp`, `one` are the slots of -0.0, +0.0 and 1.0; `lit(value)`
    returns the slot of a literal constant."""

    def __init__(self, zn: int, zp: int, one: int, lit):
        self.ops: list[tuple[int, int, int, int, int, int]] = []
        self.zn, self.zp, self.one, self.lit = zn, zp, one, lit

    def fma(self, out, a, b, c, neg=False):
        self.ops.append((FMA, out, a, b, c, int(bool(neg))))

    def rcp(self, out):
        self.ops.append((RCP, out, 0, 0, 0, 0))

    def mul(self, out, a, b):
        """S[out] = S[a] * S[b]."""
        self.fma(out, a, b, self.zn)

    def copy(self, out, a):
        self.fma(out, a, self.one, self.zn)

    def zero(self, out):
        self.fma(out, self.zp, self.zp, self.zp)

    def acc_term(self, out, first: bool, coef: float, t: int, acc: int | None = None):
        """One term of a sum accumulated left to right into S[out]: the first
        term is t, -t or c*t; later ones acc + t, acc - t or fma(c, t, acc).
        `acc` (default out) is where the running sum is read from."""
        acc = out if acc is None else acc
        if first:
            if coef == 1.0:
                self.copy(out, t)
            elif coef == -1.0:
                self.fma(out, t, self.one, self.zn, neg=True)
            else:
                self.fma(out, t, self.lit(coef), self.zn)
        else:
            if coef == 1.0:
                self.fma(out, t, self.one, acc)
            elif coef == -1.0:
                self.fma(out, t, self.one, acc, neg=True)
            else:
                self.fma(out, self.lit(coef), t, acc)

    def lu(self, plan):
        """Row-wise Doolittle factorisation in place on the LU slots (fill-in
        slots zeroed beforehand): products in plan order, then the pivot
        reciprocal or the multiply of an L entry by it."""
        diag = set(plan.diag)
        for out, w, b, e, dg in plan.ops:
            for q in range(b, e):
                pa, pb = plan.products[q]
                self.fma(out, pa, pb, out, neg=True)
            if out in diag:
                self.rcp(out)
            elif dg >= 0:
                self.mul(out, out, dg)

    def solve(self, plan, base: int):
        """(LU) x = b in place on S[base .. base + NV): unit-L forward rows
        ascending, U backward rows descending, then the reciprocal pivot."""
        nv = plan.n_var
        for i in range(nv):
            for col, slot in plan.lower[i]:
                self.fma(base + i, slot, base + col, base + i, neg=True)
        for i in range(nv - 1, -1, -1):
            for col, slot in plan.upper[i]:
                self.fma(base + i, slot, base + col, base + i, neg=True)
            self.mul(base + i, base + i, plan.diag[i])


def lu_zero_slots(plan) -> list[int]:
    """Operation outputs that start from 0 rather than from a W slot."""
    return [out for out, w, b, e, dg in plan.ops if w < 0]


def _locations(op):
    kind, out, a, b, c, _ = op
    if kind == FMA:
        return (a, b, c), (out,)
    return (out,), (out,)


def dependencies(ops) -> list[list[int]]:
    """Hazard edges of each operation on earlier operations."""
    last_write: dict = {}
    readers: dict = {}
    deps = []
    for n, op in enumerate(ops):
        reads, writes = _locations(op)
        d = set()
        for loc in reads:
            if loc in last_write:
                d.add(last_write[loc])
        for loc in writes:
            if loc in last_write:
                d.add(last_write[loc])
            d.update(r for r in readers.get(loc, ()) if r != n)
        deps.append(sorted(d))
        for loc in reads:
            readers.setdefault(loc, []).append(n)
        for loc in writes:
            last_write[loc] = n
            readers[loc] = []
    return deps


def schedule(ops, lanes: int = LANES) -> list[list[int]]:
    """Steps of at most `lanes` operations; every operation after all of its
    dependencies.  Priority: longest remaining dependency path, then program
    order."""
    n = len(ops)
    deps = dependencies(ops)
    succ = [[] for _ in range(n)]
    indeg = [len(d) for d in deps]
    for i, d in enumerate(deps):
        for j in d:
            succ[j].append(i)
    tail = [1] * n
    for i in range(n - 1, -1, -1):
        for s in succ[i]:
            tail[i] = max(tail[i], 1 + tail[s])
    ready = [(-tail[i], i) for i in range(n) if indeg[i] == 0]
    heapq.heapify(ready)
    steps = []
    done = 0
    while done < n:
        batch = [heapq.heappop(ready)[1] for _ in range(min(lanes, len(ready)))]
        if not batch:
            raise RuntimeError("dependency cycle in warp schedule")
        batch.sort()
        steps.append(batch)
        done += len(batch)
        for i in batch:
            for s in succ[i]:
                indeg[s] -= 1
                if indeg[s] == 0:
                    heapq.heappush(ready, (-tail[s], s))
    return steps


def encode(ops, steps, lanes: int = LANES) -> list[int]:
    """steps x lanes words, idle lanes marked."""
    words = []
    for batch in steps:
        row = [IDLE] * lanes
        for lane, i in enumerate(batch):
            kind, out, a, b, c, neg = ops[i]
            assert 0 <= out < IDLE and 0 <= a < 32768 and 0 <= b < 65536 and 0 <= c < 32768
            row[lane] = out | (a << 16) | (neg << 31) | (b << 32) | (c << 48) | ((kind == RCP) << 63)
        words += row
    return words


def decode(word: int) -> tuple[int, int, int, int, int, int]:
    """(kind, out, a, b, c, neg) of one word; kind 0 for an idle lane."""
    out = word & 0xFFFF
    if out == IDLE:
        return 0, out, 0, 0, 0, 0
    kind = RCP if word >> 63 else FMA
    return kind, out, (word >> 16) & 0x7FFF, (word >> 32) & 0xFFFF, (word >> 48) & 0x7FFF, (word >> 31) & 1

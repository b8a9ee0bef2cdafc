"""Static 32-lane schedules of the sparse LU and the triangular solves.

The warp-cooperative attempt runs one cell on a whole warp.  Its two
longest phases are the LU factorisation and the three triangular solves:
chains of fused multiply-adds whose order is fixed by the per-thread
kernel, and which must stay fixed so that a cell gives the same bits on
either kernel.  A level schedule that gives each lane a whole row or LU
entry idles most lanes: on SAPRC99, ~5 of 32 lanes on the LU and ~3 on the
solves.

Here every multiply-add is its own operation.  The operations are listed in
the per-thread program order:
* LU: the row-wise Doolittle operations of the reference's compact plan
  (``compact_plan.py``), each accumulating its products in plan order;
* forward solve: rows ascending, L products in plan order;
* backward solve: rows descending, U products in plan order, then the
  reciprocal-pivot multiply.

Each operation's dependencies are the read-after-write, write-after-read and
write-after-write hazards on the shared-memory slots it touches.  A list
scheduler (longest remaining path first) packs the operations into steps of
at most 32 independent ones.  Executed step by step, with a warp barrier
between steps, every slot sees the same sequence of roundings as in program
order, so the results are bit-identical.

Operation kinds, on the per-cell store S in shared memory:
  FMA  S[out] = fma(-S[a], S[b], S[out])
  MUL  S[out] = S[out] * S[b]              (times a reciprocal pivot)
  RCP  S[out] = 1 / S[out]                 (pivot; zero flags the matrix singular)
Solve programs address ``out`` and the FMA's ``b`` relative to the stage
vector; ``a`` (an LU slot) and the MUL's ``b`` (a reciprocal pivot) are
absolute.

Encoding, one 64-bit word per lane and step: bits 0-15 out, 16-31 a,
32-47 b, 48-49 kind (0 = idle lane).
"""

from __future__ import annotations

import heapq

NOP, FMA, MUL, RCP = 0, 1, 2, 3
LANES = 32


def lu_program(plan) -> list[tuple[int, int, int, int]]:
    """(kind, out, a, b) of the factorisation in per-thread order.  Slots of
    operations that do not start from a W value are zeroed beforehand."""
    diag = set(plan.diag)
    prog = []
    for out, w, b, e, dg in plan.ops:
        for q in range(b, e):
            pa, pb = plan.products[q]
            prog.append((FMA, out, pa, pb))
        if out in diag:
            prog.append((RCP, out, 0, 0))
        elif dg >= 0:
            prog.append((MUL, out, 0, dg))
    return prog


def lu_zero_slots(plan) -> list[int]:
    """Operation outputs that start from 0 rather than from a W slot."""
    return [out for out, w, b, e, dg in plan.ops if w < 0]


def solve_program(plan) -> list[tuple[int, int, int, int]]:
    """(kind, out, a, b) of (LU) x = b in place, in per-thread order."""
    nv = plan.n_var
    prog = []
    for i in range(nv):
        for col, slot in plan.lower[i]:
            prog.append((FMA, i, slot, col))
    for i in range(nv - 1, -1, -1):
        for col, slot in plan.upper[i]:
            prog.append((FMA, i, slot, col))
        prog.append((MUL, i, 0, plan.diag[i]))
    return prog


def _locations(op, relative: bool):
    """(reads, writes) of one operation as hashable slot keys."""
    kind, out, a, b = op
    if not relative:
        o, ka, kb = out, a, b
    else:
        o, ka, kb = ("r", out), ("a", a), (("r", b) if kind == FMA else ("a", b))
    if kind == FMA:
        return (o, ka, kb), (o,)
    if kind == MUL:
        return (o, kb), (o,)
    return (o,), (o,)


def dependencies(prog, relative: bool = False) -> list[list[int]]:
    """Hazard edges of each operation on earlier operations."""
    last_write: dict = {}
    readers: dict = {}
    deps = []
    for n, op in enumerate(prog):
        reads, writes = _locations(op, relative)
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


def schedule(prog, relative: bool = False, lanes: int = LANES) -> list[list[int]]:
    """Steps of at most `lanes` operations; every operation after all of its
    dependencies.  Priority: longest remaining dependency path, then program
    order."""
    n = len(prog)
    deps = dependencies(prog, relative)
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


def encode(prog, steps, lanes: int = LANES) -> list[int]:
    """steps x lanes words (idle lanes 0)."""
    words = []
    for batch in steps:
        row = [0] * lanes
        for lane, i in enumerate(batch):
            kind, out, a, b = prog[i]
            assert 0 <= out < 65536 and 0 <= a < 65536 and 0 <= b < 65536
            row[lane] = out | (a << 16) | (b << 32) | (kind << 48)
        words += row
    return words


def decode(word: int) -> tuple[int, int, int, int]:
    return (word >> 48) & 3, word & 0xFFFF, (word >> 16) & 0xFFFF, (word >> 32) & 0xFFFF

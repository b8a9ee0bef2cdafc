"""Static invariants of the device code (no GPU needed).

The reference checks its generated solvers for GPU safety by reading the
generated code (tests/python/test_gpu_safety_all_solvers.py: no heap
allocation, fully unrolled stages).  The same kind of checks here, over the
emitted headers (mkpp_gb300/generated/*.cuh) and the hand-written device
code (csrc/solver.cuh, csrc/mkpp_device.cuh):
* no heap allocation, device printf, trap or device assert;
* the emitted per-mechanism code has no while loop: every loop has a
  compile-time trip count or walks a table of known length;
* every controller loop is bounded by the attempt cap, and no device loop
  waits on memory another thread writes, so no kernel can spin forever;
* every slot a program word addresses (the cooperative stage programs, the
  table-driven adjoint and evaluation, the tangent program) lies inside the store the
  kernel gives that program, checked here from the emitted tables instead
  of by bounds checks on the device;
* the checkpoint sweeps clamp the caller's recorded-step counts to the
  checkpoint capacity.
"""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
GENERATED = sorted((ROOT / "mkpp_gb300" / "generated").glob("*.cuh"))
HANDWRITTEN = [ROOT / "mkpp_gb300" / "csrc" / f for f in ("solver.cuh", "mkpp_device.cuh")]
FORBIDDEN = (r"\bmalloc\s*\(", r"\bcalloc\s*\(", r"\brealloc\s*\(", r"\bfree\s*\(", r"\bnew\s+\w",
             r"\bdelete\b", r"\bprintf\s*\(", r"__trap\s*\(", r"\bassert\s*\(", r"\btrap\s*;",
             r"__nanosleep\s*\(")


def _code(path):
    """The file without comments and string literals."""
    text = path.read_text()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    return re.sub(r'"(?:\\.|[^"\\])*"', '""', text)


def test_the_files_exist():
    assert len(GENERATED) >= 4 and all(p.exists() for p in HANDWRITTEN)


@pytest.mark.parametrize("path", GENERATED + HANDWRITTEN, ids=lambda p: p.name)
def test_no_allocation_print_or_trap_in_device_code(path):
    code = _code(path)
    for pat in FORBIDDEN:
        assert not re.search(pat, code), (path.name, pat)


@pytest.mark.parametrize("path", GENERATED, ids=lambda p: p.name)
def test_emitted_code_has_no_while_loop(path):
    assert not re.search(r"\bwhile\s*\(", _code(path))


def test_controller_loops_are_bounded_by_the_attempt_cap():
    code = _code(ROOT / "mkpp_gb300" / "csrc" / "solver.cuh")
    loops = [m.end() for m in re.finditer(r"while\s*\(\s*ctl\.running\(\)\s*\)\s*\{", code)]
    assert loops
    for end in loops:
        body = code[end:end + 200]
        assert re.match(r"\s*if\s*\(\s*ctl\.attempts\s*>=\s*a\.max_attempts\s*\)", body), body[:120]
    # The other loops: fixed trip counts, grid-stride over cells, or the
    # persistent work loop, which ends when the queue is drained and every
    # lane's cell is done.
    whiles = len(re.findall(r"\bwhile\s*\(", code))
    assert whiles == len(loops), (whiles, len(loops))
    assert len(re.findall(r"for\s*\(\s*;\s*;\s*\)", code)) == 1
    assert "if (__ballot_sync(0xffffffffu, active) == 0u) break;" in code


@pytest.mark.parametrize("path", HANDWRITTEN, ids=lambda p: p.name)
def test_no_device_loop_polls_memory(path):
    code = _code(path)
    assert not re.search(r"\bvolatile\b", code)
    assert not re.search(r"atomicCAS\s*\(", code)


def _int_const(text, name):
    """Value of `constexpr int NAME = <literal or A + B>;` in an emitted header."""
    m = re.search(rf"constexpr int {name} = ([^;]+);", text)
    assert m, name
    expr = m.group(1).strip()
    return sum(int(t) if t.strip().isdigit() else _int_const(text, t.strip()) for t in expr.split("+"))


def _words(text, name):
    m = re.search(rf"const unsigned long long {name}\[(\d+)\] = \{{(.*?)\}};", text, re.S)
    if not m:
        return None
    words = [int(w.strip()[:-3], 0) for w in m.group(2).split(",") if w.strip()]
    assert len(words) == int(m.group(1))
    return words


def _max_slot(words):
    from mkpp_gb300.emitter import warp_schedule as ws

    top = -1
    for w in words:
        kind, out, a, b, c, _ = ws.decode(w)
        if kind == 0:
            continue
        top = max(top, out) if kind == ws.RCP else max(top, out, a, b, c)
    return top


@pytest.mark.parametrize("path", GENERATED, ids=lambda p: p.name)
def test_program_slots_lie_inside_their_stores(path):
    text = path.read_text()
    coop, adj, tlm = (_int_const(text, n) for n in ("COOP_SLOTS", "NSLOTS_ADJ", "NSLOTS_TLM"))
    sched = _words(text, "sched")
    assert sched and _max_slot(sched) < coop
    table = "TABLE_ATTEMPT = true" in text
    adj_prog, eval_prog = _words(text, "adj_prog"), _words(text, "eval_prog")
    assert (adj_prog is not None) == table and (eval_prog is not None) == table
    if table:                                     # table-driven adjoint and evaluation
        assert _max_slot(adj_prog) < adj
        assert _max_slot(eval_prog) < coop and coop == _int_const(text, "NSLOTS")
    tlm_prog = _words(text, "tlm_prog")
    assert tlm_prog and _max_slot(tlm_prog) < tlm
    assert _int_const(text, "TLM_CB") + _int_const(text, "TLM_NCONST") <= tlm
    body = text[text.index("static void tlm_step("):]
    body = body[:body.index("\n  }\n")]
    assert all(int(i) < tlm for i in re.findall(r"S\[(\d+)\] =", body))


def test_checkpoint_sweeps_read_clamped_counts():
    """The replay, adjoint and tangent sweeps read a cell's recorded-step
    count through CheckpointArgs::count (clamped to [0, cap]), since the
    device entries take the count array from the caller; only the forward
    that records the steps writes n[c] itself (0 for a cell it skips)."""
    code = _code(HANDWRITTEN[0])
    reads = re.findall(r"ck\.n\[c\][^\n;]*", code)
    assert reads == ["ck.n[c] = 0", "ck.n[c] = cnt"]
    assert len(re.findall(r"ck\.count\(c\)", code)) == 3
    assert re.search(r"int count\(size_t c\) const \{ return min\(max\(n\[c\], 0\), cap\); \}", code)

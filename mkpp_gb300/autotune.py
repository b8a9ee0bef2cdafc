"""Launch autotuner of the integrate kernels, per mechanism and GPU, cached.

    python -m mkpp_gb300.autotune saprc99 [--cells 65536] [--host-steps 2]

The knobs are those of `mkpp_set_launch_tuning` and `mkpp_set_tail_parking`:
* register variant: 2 (up to 255 registers per thread, no spills of the
  unrolled attempt) or 4 (up to 128, twice the resident warps);
* resident blocks per SM: the register variant's maximum, or fewer;
* parking threshold: attempts per host step after which the persistent
  kernel hands a cell to the warp-cooperative kernel (0: never);
* tail parking threshold (register variant 2 only): once the queue is drained
  and few cells remain on lanes, cells past it are handed over too (0: off).
A block holds 128 cells, one per thread.  The work queue hands out one cell
per lane (warp-aggregated atomics), so there is no chunk size to tune.

`tune` times every candidate on the first `cells` cells of the mechanism's
synthetic workload, integrated over `host_steps` host steps in one windowed
launch.  It keeps the fastest candidate and writes it, with the whole timing
table, to a JSON cache keyed by mechanism and GPU (name and SM count).
`apply` loads the cached choice for the current GPU and sets it.  A candidate
changes only the time: every form gives bit-identical results.
"""

from __future__ import annotations

import json
import os
import time
from dataclasses import asdict, dataclass
from pathlib import Path


@dataclass(frozen=True)
class Candidate:
    register_variant: int
    blocks_per_sm: int          # 0: as many as fit
    defer_after: int            # attempts per host step; 0: never park
    tail_after: int = 0         # tail parking threshold in attempts; 0: off


def candidates() -> list[Candidate]:
    """The search space: both register variants at full and reduced
    residency, each with parking off, at 1000 and at 3000 attempts; the
    full-residency 255-register variant also with tail parking at 300."""
    out = []
    for rv, blocks in ((2, 0), (2, 1), (4, 0), (4, 2)):
        for defer in (0, 1000, 3000):
            out.append(Candidate(rv, blocks, defer))
            if (rv, blocks) == (2, 0):
                out.append(Candidate(rv, blocks, defer, 300))
    return out


def search(measure, cands, repeats: int = 2) -> tuple[Candidate, list[dict]]:
    """Fastest candidate by `measure(candidate) -> seconds` (best of
    `repeats`).  A candidate whose measurement raises is recorded and
    skipped."""
    table = []
    best, best_s = None, float("inf")
    for c in cands:
        try:
            s = min(measure(c) for _ in range(repeats))
            err = None
        except Exception as e:  # noqa: BLE001 - a failing candidate is a result
            s, err = float("inf"), f"{type(e).__name__}: {e}"
        table.append({**asdict(c), "seconds": s, **({"error": err} if err else {})})
        if s < best_s:
            best, best_s = c, s
    if best is None:
        raise RuntimeError("no launch candidate ran")
    return best, table


def cache_path() -> Path:
    env = os.environ.get("MKPP_TUNING_CACHE")
    if env:
        return Path(env)
    return Path(os.environ.get("XDG_CACHE_HOME", Path.home() / ".cache")) / "mkpp_gb300" / "tuning.json"


def gpu_key(name: str, sms: int) -> str:
    return f"{name}/{sms}sm"


def _read(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def store(mechanism: str, gpu: str, choice: Candidate, table: list[dict], meta: dict, path: Path | None = None):
    path = path or cache_path()
    data = _read(path)
    data.setdefault(mechanism, {})[gpu] = {"choice": asdict(choice), "table": table, **meta}
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(f".tmp{os.getpid()}")
    tmp.write_text(json.dumps(data, indent=1))
    os.replace(tmp, path)


def lookup(mechanism: str, gpu: str, path: Path | None = None) -> Candidate | None:
    entry = _read(path or cache_path()).get(mechanism, {}).get(gpu)
    return Candidate(**entry["choice"]) if entry else None


def _current_gpu():
    import torch

    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return gpu_key(p.name, p.multi_processor_count)


def gpu_measure(mechanism: str, cells: int, host_steps: int):
    """A `measure` that times one windowed integrate launch (CUDA events,
    after one untimed launch per candidate) on a workload sample."""
    import numpy as np
    import torch

    from . import workloads
    from .api import DeviceSolver

    w = workloads.make(mechanism, cells)
    s = DeviceSolver(mechanism)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    conc0 = d(w.conc)
    nr = s.sizes.reactions
    ktab = torch.empty((host_steps, nr, cells), dtype=torch.float64, device="cuda")
    for h in range(host_steps):
        k, _ = s.rate_constants(conc0, d(w.temp), d(w.rho), d(w.rh), None, d(w.param_at(h)))
        ktab[h].copy_(k)
    warmed = set()

    def measure(c: Candidate) -> float:
        s.set_tuning(c.register_variant, c.blocks_per_sm, c.defer_after)
        s.set_tail_parking(c.tail_after)
        runs = 1 if c in warmed else 2
        for _ in range(runs):
            conc = conc0.clone()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            s.integrate_k(conc, ktab, w.dt, steps=host_steps, k_step_stride=nr * cells)
            b.record()
            torch.cuda.synchronize()
        warmed.add(c)
        return a.elapsed_time(b) * 1e-3

    return measure


def tune(mechanism: str, cells: int = 65536, host_steps: int = 2, path: Path | None = None) -> Candidate:
    gpu = _current_gpu()
    t0 = time.time()
    best, table = search(gpu_measure(mechanism, cells, host_steps), candidates())
    store(mechanism, gpu, best, table, {"cells": cells, "host_steps": host_steps,
                                       "tuning_seconds": time.time() - t0}, path)
    return best


def apply(mechanism: str, path: Path | None = None) -> Candidate | None:
    """Set the cached choice for this mechanism on the current GPU (None and
    no change if there is none)."""
    from .api import DeviceSolver

    c = lookup(mechanism, _current_gpu(), path)
    if c is not None:
        s = DeviceSolver(mechanism)
        s.set_tuning(c.register_variant, c.blocks_per_sm, c.defer_after)
        s.set_tail_parking(c.tail_after)
    return c


def main(argv=None) -> int:
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("mechanism")
    ap.add_argument("--cells", type=int, default=65536)
    ap.add_argument("--host-steps", type=int, default=2)
    a = ap.parse_args(argv)
    best = tune(a.mechanism, a.cells, a.host_steps)
    print(json.dumps({"mechanism": a.mechanism, "choice": asdict(best), "cache": str(cache_path())}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())

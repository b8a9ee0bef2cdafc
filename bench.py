#!/usr/bin/env python
"""SAPRC99 cell-solves/s on GB300 (FP64 Rosenbrock, rtol 1e-3, atol 1).

Workload: 262144 synthetic SAPRC99 cells integrated over 24 host steps of
600 s (seeded draws, see mkpp_gb300/workloads.py).  One bench step is that
whole integration: restore the initial state, then for each host step compute
the rate constants from the hour's photolysis and integrate every cell with
the persistent work-queue kernel.  The 24 host steps are captured once as a
CUDA graph and each step is one graph launch.  value = cells * host steps /
step time (cell-solves/s, summed over ranks).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The JSON line also carries: e2e (the same run through the host-buffer C ABI
mkpp_integrate, copies included), roofline (FP64 pipe of the integrate kernel
against a live DFMA probe), cpu_baseline, the plain one-thread-per-cell
per-launch form for comparison, clocks sampled during the timed region, and
gpu_launches.
"""

from __future__ import annotations

import argparse
import contextlib
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

# Thread placement of the CPU legs (the reference solver's OpenMP loop):
# spread over all cores, one thread per core, as the reference's benchmark
# recipe runs it.  Read once, when the OpenMP runtime starts.
os.environ.setdefault("OMP_PROC_BIND", "spread")
os.environ.setdefault("OMP_PLACES", "cores")

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SAPRC99 cell-solves/s on 1 GB300 at rtol 1e-3"

# DRAM read + write bytes of integrate_persistent_kernel per attempt, from one
# ncu capture of the capped case (python bench.py --bulk-only --bulk-cells
# 19456 --bulk-attempts 20): 32.79 GB over 389120 attempts.
DRAM_BYTES_PER_ATTEMPT = {"saprc99": 84.3e3}


def metric_for(mechanism: str) -> str:
    """The metric's name for a workload: METRIC itself for SAPRC99, the same
    wording with the mechanism's name for the others."""
    return METRIC if mechanism == "saprc99" else METRIC.replace("SAPRC99", mechanism.upper(), 1)


UNIT = "cell-solves/s"


T_START = time.time()


def log(msg):
    """Progress on stderr (the JSON result line is the only stdout output)."""
    print(f"[bench {time.time() - T_START:7.1f}s] {msg}", file=sys.stderr, flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", default="saprc99")
    ap.add_argument("--cells", type=int, default=None)
    ap.add_argument("--host-steps", type=int, default=None)
    ap.add_argument("--cpu-cells", type=int, default=None,
                    help="cells in the bounded CPU sample (default max(4096, 64 x threads): every thread gets "
                         "at least one of the reference's 64-cell chunks per host step)")
    ap.add_argument("--cpu-chunk", type=int, default=64,
                    help="cells per static OpenMP chunk of the reference CPU solver (the reference's 64); a "
                         "smaller chunk keeps every thread busy on a sample of fewer than 64 cells per thread")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--max-attempts", type=int, default=20000)
    ap.add_argument("--order", type=int, default=1, help="hand out cells most-expensive-first (previous window)")
    ap.add_argument("--forms-cells", type=int, default=65536, help="cells of the plain-vs-persistent comparison")
    ap.add_argument("--forms-host-steps", type=int, default=2, help="host steps of that comparison")
    ap.add_argument("--adjoint-cells", type=int, default=None,
                    help="cells of the adjoint/forward measurement (default: 65536 for one 3600 s integrate(); "
                         "every cell for the window gradient)")
    ap.add_argument("--adjoint-window", type=int, default=None,
                    help="1: gradient of the whole window (every host step, two-level checkpoints, "
                         "WindowGradient); 0: of one 3600 s integrate().  Default: the window for ts1")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--adjoint-check-cells", type=int, default=256,
                    help="cells of the adjoint's accuracy check against central differences through the "
                         "recorded steps (0: skip)")
    ap.add_argument("--tangent", type=int, default=0,
                    help="also time the tangent sweep over the adjoint section's checkpoints (mkpp_gpu_tangent)")
    ap.add_argument("--tail-after", type=int, default=None,
                    help="tail parking threshold in attempts for every integrate launch (mkpp_set_tail_parking; 0 off)")
    ap.add_argument("--e2e-cost-order", type=int, default=1,
                    help="e2e handle hands out the previous call's most expensive cells first (mkpp_set_cost_order)")
    ap.add_argument("--bulk-cells", type=int, default=77824,
                    help="cells of the bulk-rate section (every cell capped at --bulk-attempts attempts)")
    ap.add_argument("--bulk-attempts", type=int, default=20)
    ap.add_argument("--bulk-defer", type=int, default=0,
                    help="park each cell for the warp-cooperative kernel after this many attempts (0: never); "
                         "1 with few cells measures the cooperative kernel's attempt latency")
    ap.add_argument("--tune", type=int, default=1,
                    help="1: the warm-up windows compare launch configurations (default, tail parking, split "
                         "launch) and the fastest is timed; 0: time the flags' configuration")
    ap.add_argument("--split", default="auto",
                    help="split launch of the window (mkpp_set_split_launch): 'auto' plans it from the first "
                         "warm-up window's attempt counts and keeps it only if a warm-up window with it beats one "
                         "without, 'off', or CELLS:SMS")
    ap.add_argument("--bulk-only", action="store_true",
                    help="run only the bulk-rate section (a small case for profilers) and print its JSON")
    return ap.parse_args()


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        load = [r for r in rows if r[2] > 200.0] or rows
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in load for n, v in zip(names, r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "power_w_max": max(r[2] for r in rows)}


def dist_setup(args):
    """One process per GPU (torchrun); NCCL for our arm, gloo for the CPU
    reference arm.  Cells shard with no data-path collective
    (mkpp_gb300/shard.py)."""
    from mkpp_gb300 import shard

    env = shard.rank_env()
    shard.init(env, "nccl" if args.impl == "ours" else "gloo")
    return env.world, env.rank, env.local


def barrier(world):
    from mkpp_gb300 import shard

    shard.barrier()


@contextlib.contextmanager
def optional_section(result: dict, name: str, guard: bool = True):
    """A secondary measurement: if it raises (and guard is set), its key in
    the JSON line records the error instead of the run losing the headline
    numbers already measured.  Unguarded where ranks must stay in step."""
    if not guard:
        yield
        return
    try:
        yield
    except Exception as e:  # noqa: BLE001
        result[name] = {"error": f"{type(e).__name__}: {e}"}
        log(f"{name}: failed: {type(e).__name__}: {e}")


def max_over_ranks(x: float, world: int) -> float:
    from mkpp_gb300 import shard

    return shard.max_over_ranks(x)


# ---------------------------------------------------------------------------
def bulk_rate(mechanism: str, cells: int, attempts: int, stream=None, defer: int = 0) -> dict:
    """Attempt throughput of the persistent kernel with every lane busy: the
    first `cells` cells of the workload (first host step) with every cell
    capped at `attempts` attempts, so no cell finishes early and there is no
    tail; nothing is parked unless `defer` > 0, which parks every cell after
    that many attempts (this sets the process's parking threshold, so it runs
    last).  Two launches, the second timed with CUDA events on the
    launching stream.  Explains the window's roofline fraction: the gap
    between the two is the tail."""
    import torch

    from mkpp_gb300 import workloads
    from mkpp_gb300.api import DeviceSolver
    from mkpp_gb300.emitter.plan import flops_per_attempt, load

    w = workloads.make(mechanism, cells)
    s = DeviceSolver(mechanism)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    conc0 = d(w.conc)
    stream = stream or torch.cuda.current_stream()
    with torch.cuda.stream(stream):
        ktab, status = s.rate_constants(conc0, d(w.temp), d(w.rho), d(w.rh), None, d(w.param))
        s.set_tuning(defer_after=defer)
        for rep in range(2):
            conc = conc0.clone()
            st = status.clone()
            acc = torch.zeros(cells, dtype=torch.int32, device="cuda")
            rej = torch.zeros_like(acc)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            s.integrate_k(conc, ktab, w.dt, max_attempts=attempts, mode="persistent", status=st, accepted=acc,
                          rejected=rej)
            b.record(stream)
            stream.synchronize()
    att = int((acc + rej).sum())
    ms = a.elapsed_time(b)
    flops = flops_per_attempt(load(mechanism))["total"]
    return {"cells": cells, "attempt_cap": attempts, "defer_after": defer, "attempts": att, "ms": ms,
            "attempts_per_s": att / (ms * 1e-3), "tflops": att * flops / (ms * 1e-3) / 1e12}


def adjoint_accuracy_section(mechanism, raw, var_rows, solver, conc0, temp, rho, rh, param, seed, cells,
                             max_attempts, checkpoints_cls, eps=1e-6) -> dict:
    """Accuracy of the discrete adjoint on the bench's own cells, at the
    adjoint section's setting (one 3600 s integrate(), loss sum (O3 - O3t)^2).
    Two directions: one in the variable species' initial concentrations and
    one in the rate constants, each component its value with a random sign.
    Along each, the adjoint's directional derivative g.u against central
    differences through the same recorded accepted steps (the replay), at
    relative steps eps and 10 eps.  Only the GPU path runs here.  Per cell:
    the relative error |fd - g.u| / max(|fd|, |g.u|) at eps, and the
    differences' own noise |fd(eps) - fd(10 eps)| / max(...), since on
    ill-conditioned cells round-off in the replay sets the differences'
    accuracy; `frac_consistent` counts the cells whose error is within 1e-4
    or within twice that noise.  Over the cells that end with status 0 and
    finite values."""
    import torch

    f64 = torch.float64
    dev = conc0.device
    m = min(cells, conc0.shape[1])
    c0 = conc0[:, :m].contiguous()
    k, st_in = solver.rate_constants(c0, temp[:m].contiguous(), rho[:m].contiguous(), rh[:m].contiguous(),
                                     None, param[:, :m].contiguous())
    ck = checkpoints_cls(mechanism, m, 1536, dev)
    c = c0.clone()
    ck.forward(c, k, 3600.0, seed, max_attempts)
    o3 = raw["species"].index("O3")
    gen = torch.Generator(device="cpu").manual_seed(2718)
    target = c[o3] * torch.exp(0.2 * torch.randn(m, generator=gen, dtype=f64)).to(dev)
    lam = torch.zeros_like(c)
    lam[o3] = 2.0 * (c[o3] - target)
    gc, gk = ck.adjoint(k, lam)

    def loss(x):
        return (x[o3] - target) ** 2

    def signs(shape):
        return (torch.randint(0, 2, shape, generator=gen) * 2 - 1).to(device=dev, dtype=f64)

    mask = torch.zeros((c0.shape[0], 1), dtype=f64, device=dev)
    mask[list(var_rows)] = 1.0
    uc = c0.abs() * signs(c0.shape) * mask
    uk = k.abs() * signs(k.shape)
    fd_c, fd_k = [], []
    for e in (eps, 10 * eps):
        cp, cm = c0 + e * uc, c0 - e * uc
        ck.replay(cp, k)
        ck.replay(cm, k)
        fd_c.append((loss(cp) - loss(cm)) / (2 * e))
        cp, cm = c0.clone(), c0.clone()
        ck.replay(cp, k + e * uk)
        ck.replay(cm, k - e * uk)
        fd_k.append((loss(cp) - loss(cm)) / (2 * e))
    ad_c, ad_k = (gc * uc).sum(0), (gk * uk).sum(0)
    if dev.type == "cuda":
        torch.cuda.synchronize()
    ok = ((ck.status == 0) & (st_in == 0)).cpu().numpy()

    def rel(x, y):
        return np.abs(x - y) / np.maximum(np.maximum(np.abs(x), np.abs(y)), 1e-300)

    def stats(fd, ad):
        f1, f2, ad = fd[0].cpu().numpy(), fd[1].cpu().numpy(), ad.cpu().numpy()
        use = ok & np.isfinite(f1) & np.isfinite(f2) & np.isfinite(ad)
        if not use.any():
            return {"cells": 0}
        err, noise = rel(f1, ad)[use], rel(f1, f2)[use]
        return {"cells": int(use.sum()), "median_rel_error": float(np.median(err)),
                "p90_rel_error": float(np.percentile(err, 90)), "max_rel_error": float(err.max()),
                "median_difference_noise": float(np.median(noise)),
                "frac_within_1e-4": float((err <= 1e-4).mean()),
                "frac_consistent": float((err <= np.maximum(1e-4, 2 * noise)).mean())}

    return {"config": f"first {m} cells, one 3600 s integrate(), the adjoint section's loss; central differences "
                      f"(relative steps {eps:g} and {10 * eps:g}, random signs) through the recorded accepted steps",
            "initial_concentrations": stats(fd_c, ad_c), "rate_constants": stats(fd_k, ad_k),
            "cells_status_ok": int(ok.sum())}


def adjoint_window_section(w, hs, conc0, ktab, seed, args, stream, window_ms) -> dict:
    """Gradient of L = sum_c (O3_c(end) - O3t_c)^2 over the whole window (every
    host step, each with its own rate constants) with respect to the initial
    concentrations and the rate constants of every host step, through
    WindowGradient: the forward keeps the host-step boundary states (one
    persistent launch per host step); the backward recomputes each host step
    of each chunk of cells with checkpoints at its accepted steps and sweeps
    it in reverse.  Reported: backward / forward time, also against the
    timed window's time for the same cells."""
    import torch

    from mkpp_gb300.adjoint import WindowGradient
    from mkpp_gb300.api import DeviceSolver, sizes
    from mkpp_gb300.emitter.plan import load_raw

    raw = load_raw(w.mechanism)
    n = w.ncells
    na = min(n, args.adjoint_cells or n)
    nv = sizes(w.mechanism).variable
    cap = 1024
    # Level-2 checkpoints of one chunk: at most 60 GB.
    chunk = max(128, min(na, int(60e9 // (cap * (nv + 1) * 8)) // 128 * 128))
    dev = conc0.device
    k = ktab if na == n else ktab[:, :, :na].contiguous()
    wg = WindowGradient(w.mechanism, na, hs, dev, cap=cap, chunk=chunk)
    solver = DeviceSolver(w.mechanism)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    with torch.cuda.stream(stream):
        conc = conc0[:, :na].clone()
        ev[0].record(stream)
        wg.forward(conc, k, w.dt, seed, args.max_attempts, solver=solver)
        ev[1].record(stream)
        stream.synchronize()
        o3 = raw["species"].index("O3")
        rng = torch.Generator(device="cpu").manual_seed(2718)
        target = conc[o3] * torch.exp(0.2 * torch.randn(na, generator=rng, dtype=torch.float64)).to(dev)
        lam = torch.zeros_like(conc)
        lam[o3] = 2.0 * (conc[o3] - target)
        ev[2].record(stream)
        gc, gk = wg.backward(k, lam)
        ev[3].record(stream)
        stream.synchronize()
    fms, bms = ev[0].elapsed_time(ev[1]), ev[2].elapsed_time(ev[3])
    st = wg.status.cpu().numpy()
    fin = (torch.isfinite(gc).all(0) & torch.isfinite(gk).all(0).all(0)).double().mean().item()
    out = {
        "config": f"first {na} cells, {hs} host steps of {w.dt:g} s, loss sum (O3 - O3t)^2, O3t log-normal "
                  f"sigma 0.2; two-level checkpoints (host-step boundaries; accepted steps of {chunk}-cell "
                  f"chunks, cap {cap})",
        "forward_ms": fms, "backward_ms": bms, "adjoint_over_forward": bms / fms,
        "adjoint_over_window_forward": bms / (window_ms * na / n),
        "cell_status_counts": np.bincount(st, minlength=6).tolist(),
        "gradients": f"dL/dC0 for all species and dL/dk for all {len(raw['reactions'])} reactions of every "
                     f"host step, FP64",
        "finite_gradients_frac": fin,
    }
    del wg, gc, gk
    torch.cuda.empty_cache()
    return out


def cpu_sample_cells(args, threads: int) -> int:
    """Cells of the CPU sample: at least 4096, and at least one 64-cell chunk
    of the reference's static OpenMP schedule per thread."""
    return args.cpu_cells or max(4096, 64 * threads)


def cpu_runner(mechanism: str):
    """The reference's own CPU solver built here (kind "reference"), else the
    oracle port (kind "port")."""
    try:
        from oracle import ref_build

        ref = ref_build.load(mechanism)
        if ref is None and mechanism in ref_build.ON_DEMAND + tuple(ref_build.VARIANTS):
            ref = ref_build.ensure(mechanism)   # compiled here from its generated headers
    except Exception:
        ref = None
    if ref is not None:
        return "reference", ref
    from oracle.oracle import Oracle

    return "port", Oracle(mechanism)


def cpu_integrate(runner, sub, conc, first: int, last: int, threads: int, chunk: int = 64) -> float:
    """Host steps [first, last) of every cell of `sub`, in place on conc;
    returns the seconds.  One OpenMP parallel region per host step, as the
    reference's host loop calls its dispatcher once per host step."""
    extra = {"chunk": chunk} if chunk != 64 and hasattr(runner, "np_") else {}
    params = [sub.param_at(s) for s in range(first, last)]
    t0 = time.perf_counter()
    for par in params:
        runner.integrate(conc, sub.dt, temp=sub.temp, rho=sub.rho, rh=sub.rh, param=par, nthreads=threads,
                         **extra)
    return time.perf_counter() - t0


def cpu_reference_sample(w, cells: int, host_steps: int, threads: int, chunk: int = 64, out=None):
    """Time the CPU implementation on the first `cells` cells of the workload,
    all host steps (the end state goes to `out` when given)."""
    sub = w.subset(cells)
    kind, runner = cpu_runner(sub.mechanism)
    conc = sub.conc.copy()
    el = cpu_integrate(runner, sub, conc, 0, host_steps, threads, chunk)
    if out is not None:
        out.append(conc)
    return kind, cells * host_steps / el, el


def parity_against(got, ref, raw) -> dict:
    """The GPU window's end state against the CPU solver's on the same cells:
    per species |got - ref| in units of rtol |ref| + atol (the tolerance),
    and relative to |ref| + atol."""
    atol = np.array(raw["atol"])[:, None]
    rtol = np.array(raw["rtol"])[:, None]
    both = np.isfinite(got).all(axis=0) & np.isfinite(ref).all(axis=0)
    d = np.abs(got - ref)[:, both]
    r = np.abs(ref)[:, both]
    tol_units = d / (rtol * r + atol)
    per_cell = tol_units.max(axis=0) if both.any() else np.zeros(0)
    return {"cells": int(got.shape[1]), "both_finite": int(both.sum()),
            "nonfinite_same_cells": bool(np.array_equal(~np.isfinite(got).all(axis=0),
                                                        ~np.isfinite(ref).all(axis=0))),
            "max_error_tolerance_units": float(tol_units.max()) if both.any() else None,
            "median_relative_error": float(np.median(d / (r + atol))) if both.any() else None,
            "cells_within_tolerance_frac": float((per_cell <= 1.0).mean()) if both.any() else None,
            "cells_within_10x_tolerance_frac": float((per_cell <= 10.0).mean()) if both.any() else None}


def run_reference(args, world, rank):
    from mkpp_gb300 import workloads

    if rank != 0:
        return
    w = workloads.make(args.workload, args.cells)
    hs = args.host_steps or w.host_steps
    threads = os.cpu_count() or 1
    cells = min(cpu_sample_cells(args, threads), w.ncells)
    kind, runner = cpu_runner(w.mechanism)
    # Warm-up steps: one host step of one chunk per thread (at most the sample).
    warm = w.subset(min(args.cpu_chunk * threads, cells))
    for _ in range(args.warmup):
        cpu_integrate(runner, warm, warm.conc.copy(), 0, 1, threads, args.cpu_chunk)
    # Timed steps: together they integrate one whole window (all host steps)
    # of the sample, step i taking host steps [hs i / K, hs (i + 1) / K), so
    # the run stays bounded whatever K is while the sample keeps the cost mix
    # of the whole window (the first host step is the stiffest).  With more
    # steps than host steps, windows repeat from the initial state.
    sub = w.subset(cells)
    windows = -(-args.steps // hs)
    passes = windows * hs
    conc = sub.conc.copy()
    total = 0.0
    for i in range(args.steps):
        for x in range(passes * i // args.steps, passes * (i + 1) // args.steps):
            if x % hs == 0:
                conc = sub.conc.copy()
            total += cpu_integrate(runner, sub, conc, x % hs, x % hs + 1, threads, args.cpu_chunk)
    value = cells * passes / total
    ms = total / args.steps * 1e3
    sample = (f"first {cells} of {w.ncells} cells x {hs} host steps of {w.dt:g} s"
              + (f" ({windows} windows)" if windows > 1 else "") + f", split over the {args.steps} timed steps; "
              f"OpenMP static chunks of {args.cpu_chunk} cells, OMP_PROC_BIND={os.environ.get('OMP_PROC_BIND')}, "
              f"OMP_PLACES={os.environ.get('OMP_PLACES')}")
    line = {
        "impl": "reference", "metric": metric_for(w.mechanism), "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(w, hs),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample,
                         "seconds": total},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


L2_BYTES = 129 * 2**20            # GB300 L2
L2_FLUSH_BYTES = 512 * 2**20      # written between timed steps when the inputs fit in L2


def window_input_bytes(w, hs):
    """Bytes one window reads: concentrations, runtime parameters and the
    rate-constant table of every host step."""
    from mkpp_gb300.emitter.plan import load_raw

    raw = load_raw(w.mechanism)
    return 8 * w.ncells * (len(raw["species"]) + hs * (raw["num_reactions"] + raw["num_rate_parameters"]))


def inputs_exceed_l2(w, hs):
    return window_input_bytes(w, hs) > 2 * L2_BYTES


def workload_config(w, hs):
    from mkpp_gb300.emitter.plan import load_raw

    raw = load_raw(w.mechanism)
    mb = window_input_bytes(w, hs) / 1e6
    l2 = (f"inputs larger than L2 ({mb:.0f} MB of concentrations, parameters and rate constants per window)"
          if inputs_exceed_l2(w, hs) else
          f"L2 flushed before every timed step by a {L2_FLUSH_BYTES >> 20} MiB write (the window's {mb:.1f} MB of "
          "inputs fit in L2)")
    return {"workload": f"{w.mechanism}: {w.ncells} cells x {hs} host steps of {w.dt:g} s, "
                        f"{raw['tableau']['name']}, rtol {raw['rtol'][0]:g}, atol {raw['atol'][0]:g}",
            "mechanism": w.mechanism, "cells_per_gpu": w.ncells, "host_steps": hs, "dt_s": w.dt,
            "tableau": raw["tableau"]["name"],
            "form": "CUDA graph per window: rate constants of every host step, then one persistent work-queue "
                    "launch carrying each cell through all host steps (cells ordered by the previous window's cost)",
            "l2": l2}


# ---------------------------------------------------------------------------
def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import torch

    from mkpp_gb300 import workloads
    from mkpp_gb300.api import MKPP_SUCCESS, DeviceSolver, MechanismContext, load_library
    from mkpp_gb300.emitter.plan import flops_per_attempt, load, load_raw

    torch.cuda.set_device(local)
    if args.bulk_only:
        print(json.dumps({"bulk": bulk_rate(args.workload, args.bulk_cells, args.bulk_attempts,
                                            defer=args.bulk_defer)}), flush=True)
        return
    dev = torch.device("cuda", local)
    from mkpp_gb300 import shard

    w = workloads.make(args.workload, args.cells, seed=shard.shard_seed(workloads.SEED, rank))
    hs = args.host_steps or w.host_steps
    n = w.ncells
    raw = load_raw(w.mechanism)
    plan = load(w.mechanism)
    lib = load_library(w.mechanism)
    solver = DeviceSolver(w.mechanism)
    # Tail parking threshold the runs use unless the tuning below picks
    # another: the flag, else the library's default (MKPP_TAIL_AFTER or 300).
    lib_tail = args.tail_after if args.tail_after is not None else int(os.environ.get("MKPP_TAIL_AFTER", "300"))
    solver.set_tail_parking(lib_tail)
    NS, NR, NP = solver.sizes.species, solver.sizes.reactions, solver.sizes.rate_parameters
    seed = float(raw["initial_step_seed"])

    f64 = torch.float64
    conc0 = torch.from_numpy(w.conc).to(dev)
    conc = conc0.clone()
    temp = torch.from_numpy(w.temp).to(dev)
    rho = torch.from_numpy(w.rho).to(dev)
    rh = torch.from_numpy(w.rh).to(dev)
    params = torch.from_numpy(np.stack([w.param_at(s) for s in range(hs)])).to(dev)
    # Rate constants of every host step of the window: [hs][NR][n].
    ktab = torch.empty((hs, NR, n), dtype=f64, device=dev)
    status = torch.zeros(n, dtype=torch.int32, device=dev)
    acc = torch.zeros(n, dtype=torch.int32, device=dev)
    rej = torch.zeros(n, dtype=torch.int32, device=dev)
    order = torch.arange(n, dtype=torch.int32, device=dev)
    ws_bytes = int(lib.mkpp_gpu_workspace_bytes(C.c_size_t(n)))
    ws = torch.zeros(max(ws_bytes, 256), dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sp = C.c_void_p(stream.cuda_stream)
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    def check(rc, what):
        if rc != MKPP_SUCCESS:
            raise RuntimeError(f"{what} failed: {rc}")

    def rates():
        for s in range(hs):
            check(lib.mkpp_gpu_rate_constants(C.c_size_t(n), p(conc), p(temp), p(rho), p(rh), None, p(params[s]),
                                              C.c_size_t(NP), p(ktab[s]), p(status) if s == 0 else None, sp),
                  "rate constants")

    def window(events=None):
        """The persistent form: all host steps of every cell in one launch,
        cells handed out most expensive first (cost of the previous window)."""
        conc.copy_(conc0)
        rates()
        if events is not None:
            events[0].record(stream)
        check(lib.mkpp_gpu_integrate_k(C.c_size_t(n), p(conc), p(ktab), C.c_size_t(NR * n), hs, C.c_double(w.dt),
                                       C.c_double(seed), args.max_attempts, 1, p(order) if args.order else None,
                                       p(status), p(acc), p(rej), p(ws), C.c_size_t(ws.numel()), sp), "integrate")
        if events is not None:
            events[1].record(stream)
        if args.order:
            order.copy_(torch.argsort(acc + rej, descending=True).to(torch.int32))

    # Launch tuning in the warm-up windows.  Window 0 runs in cell order and
    # gives every cell's attempt count; each later warm-up window (now in
    # cost order) runs one candidate launch configuration, and the fastest
    # is the one timed:
    #   default   the library's settings (tail parking after 300 attempts);
    #   tail      tail parking after 300 attempts, where the flags turned it
    #             off (mkpp_set_tail_parking);
    #   split     the split launch (mkpp_set_split_launch): the 0.1% most
    #             expensive cells of the previous window on whole warps of
    #             one reserved SM per 25 of them (SAPRC99, 262144 cells: 262
    #             cells on 10 SMs; measured there, 200 cells on 8 SMs took
    #             the window from 38.3 s to 32.3 s, and a model-planned 23
    #             cells on 1 SM lengthened it to 41.3 s).
    # Every candidate gives bit-identical results.  --tune 0 times the
    # configuration the flags give, unchanged.
    tune_info = {"tuned": bool(args.tune and args.order and args.warmup >= 2)}
    fixed_split = (0, 0) if args.split in ("auto", "off") else tuple(int(x) for x in args.split.split(":"))
    if args.split == "auto":
        k = max(1, round(n * 1e-3))
        auto_split = (k, max(1, min(16, round(k / 25))))
    else:
        auto_split = fixed_split

    def apply_config(cfg):
        solver.set_tail_parking(cfg["tail"])
        solver.set_split_launch(*cfg["split"])

    configs = [{"name": "default", "tail": lib_tail, "split": (0, 0) if tune_info["tuned"] else fixed_split}]
    if tune_info["tuned"]:
        if lib_tail == 0:
            configs.append({"name": "tail", "tail": 300, "split": (0, 0)})
        if args.split != "off":
            configs.append({"name": "split", "tail": 0, "split": auto_split})
    ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    kernel_ms = []
    cfg_of = []            # the configuration each warm-up window ran
    chosen = configs[0]
    apply_config(chosen)
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            if tune_info["tuned"] and i >= 1:
                # the likely winners first: with the default three warm-up
                # windows only two candidates get a window
                priority = {"split": 0, "tail": 1, "default": 2}
                pending = sorted((c for c in configs if "ms" not in c), key=lambda c: priority[c["name"]])
                if pending:
                    chosen = pending[0]
                else:
                    chosen = min(configs, key=lambda c: c["ms"])
                apply_config(chosen)
            window(ev)
            stream.synchronize()
            kernel_ms.append(ev[0].elapsed_time(ev[1]))
            cfg_of.append(chosen["name"])
            if i >= 1 and "ms" not in chosen:
                chosen["ms"] = kernel_ms[-1]
            log(f"warm-up window {i}: integrate {kernel_ms[-1]:.0f} ms ({chosen['name']})")
        if tune_info["tuned"]:
            measured = [c for c in configs if "ms" in c]
            chosen = min(measured, key=lambda c: c["ms"]) if measured else configs[0]
            apply_config(chosen)
    tune_info["candidates_ms"] = {c["name"]: c.get("ms") for c in configs}
    tune_info["chosen"] = {"name": chosen["name"], "tail_after": chosen["tail"], "split_cells_sms": list(chosen["split"])}
    split = tuple(chosen["split"])
    timed_cfg_ms = [ms for i, (ms, name) in enumerate(zip(kernel_ms, cfg_of)) if i >= 1 and name == chosen["name"]]
    if not timed_cfg_ms:
        timed_cfg_ms = kernel_ms[1:] or kernel_ms
    # Capture the window: hs rate-constant launches, the persistent integrate
    # launch and, with parking enabled, the cooperative launch (which finds no
    # parked cell: no cell of a 24-step window reaches 24 x 3000 attempts).
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(g, stream=stream):
            window()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # Inputs that fit in L2 would be served from it by the previous step's
    # reads: then every timed step is preceded by a write larger than L2,
    # outside that step's events.
    flush = None if inputs_exceed_l2(w, hs) else torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks, torch.cuda.stream(stream):
        if flush is None:
            start.record(stream)
            for _ in range(args.steps):
                g.replay()
            end.record(stream)
            torch.cuda.synchronize()
            timed_ms = start.elapsed_time(end)
        else:
            step_ev = []
            for i in range(args.steps):
                flush.fill_(i & 0xff)
                e = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                e[0].record(stream)
                g.replay()
                e[1].record(stream)
                step_ev.append(e)
            torch.cuda.synchronize()
            timed_ms = sum(a.elapsed_time(b) for a, b in step_ev)
    barrier(world)
    el_ms = max_over_ranks(timed_ms, world) / args.steps
    log(f"timed: {el_ms:.0f} ms per window")
    # End state of the timed window's first cells, for the parity check
    # against the CPU reference solver on the same cells (cpu_baseline).
    window_end = conc[:, :min(n, cpu_sample_cells(args, os.cpu_count() or 1))].cpu().numpy()
    # The later sections run with the library's defaults and the flags.
    solver.set_split_launch(0, 0)
    solver.set_tail_parking(lib_tail)
    clk = clocks.summary()
    cell_solves = shard.sum_over_ranks(n * hs)
    value = cell_solves / (el_ms * 1e-3)

    # Work counters of the (deterministic) window just timed.
    att = (acc + rej).cpu().numpy().astype(np.int64)
    st_h = status.cpu().numpy()
    attempts = int(att.sum())
    fpa = flops_per_attempt(plan)
    flops_run = attempts * fpa["total"]
    kernel_avg_ms = statistics.mean(timed_cfg_ms) if kernel_ms else float("nan")
    achieved = flops_run / (kernel_avg_ms * 1e-3) / 1e12 if kernel_ms else None

    # Live FP64 FMA peak (DFMA probe on this GPU).
    probe = C.CDLL(str(ROOT / "mkpp_gb300" / "lib" / "libgb300_fp64_probe.so"))
    probe.mkpp_probe_fp64_fma.restype = C.c_double
    probe.mkpp_probe_fp64_fma.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    pout = torch.zeros(sms * 8, dtype=f64, device=dev)
    best = 0.0
    with torch.cuda.stream(stream):
        for _ in range(4):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fl = probe.mkpp_probe_fp64_fma(p(pout), sms * 8, 256, 2000, sp)
            b.record(stream)
            stream.synchronize()
            best = max(best, fl / (a.elapsed_time(b) * 1e-3) / 1e12)
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    peaks = json.loads(peaks_path.read_text()) if peaks_path.exists() else {}

    result = {
        "metric": metric_for(w.mechanism), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(w, hs),
        "gpu_launches": args.steps * (hs + 1 + (int(os.environ.get("MKPP_DEFER_AFTER", "3000")) > 0
                                                or chosen["tail"] > 0)),
        "launch": {"register_variant": os.environ.get("MKPP_REGISTER_VARIANT", "2"),
                   "blocks_per_sm": os.environ.get("MKPP_BLOCKS_PER_SM", "max"),
                   "defer_after_per_host_step": os.environ.get("MKPP_DEFER_AFTER", "3000"), "cost_order": bool(args.order),
                   "tail_after": chosen["tail"],
                   "max_attempts_per_call": args.max_attempts, "tuning": tune_info},
        "clocks": clk,
        "work": {"attempts_per_cell_solve": attempts / (n * hs), "flops_per_attempt": fpa["total"],
                 "attempts_per_cell_window_pct": {q: float(np.percentile(att, q)) for q in (50, 90, 99, 100)},
                 "cell_status_counts": np.bincount(st_h, minlength=5).tolist(),
                 # value counting only the cells that end finite (status 4 is
                 # a non-finite result, as the oracle gives for the same cells)
                 "value_finite_cells_only": float((st_h != 4).sum()) * hs / (el_ms * 1e-3)},
        "roofline": {
            "bound": "fp64", "achieved": achieved, "peak": best, "unit": "TFLOP/s",
            "frac": (achieved / best) if achieved and best else None,
            "peak_source": "measured live: DFMA probe (csrc/probe.cu) on this GPU",
            # the integrate call's launches, timed together by the events
            "kernel": (("integrate_split_kernel" if split != (0, 0) else "integrate_persistent_kernel")
                       + (" + integrate_coop_kernel" if chosen["tail"] > 0 or
                          int(os.environ.get("MKPP_DEFER_AFTER", "3000")) > 0 else "")),
            "launch_ms_avg": kernel_avg_ms,
            "algorithmic_flops_per_launch": flops_run,
            # DRAM bytes of the integrate kernel per launch: the ncu capture of
            # the capped case (19456 cells x 20 attempts, dram__bytes_read +
            # dram__bytes_write per attempt) scaled by this window's attempts.
            "traffic": (attempts * DRAM_BYTES_PER_ATTEMPT[w.mechanism]
                        if w.mechanism in DRAM_BYTES_PER_ATTEMPT else None),
            "traffic_unit": "bytes per launch",
            "traffic_source": ("ncu, capped case, scaled by attempts (profiles/integrate_persistent_saprc99.md)"
                               if w.mechanism in DRAM_BYTES_PER_ATTEMPT else None),
            "hbm_peak_gbs": peaks.get("hbm_gbs"),
        },
    }

    if rank == 0 and not args.no_plain:
        with optional_section(result, "forms", True):
            # Forms on a sub-configuration (first forms_cells cells, first
            # forms_host_steps host steps): plain = one launch per host step, one
            # thread per cell, no queue; persistent = the window form above.
            fn, fh = min(n, args.forms_cells), min(hs, args.forms_host_steps)
            sub = conc0[:, :fn].contiguous()
            c2 = sub.clone()
            k2 = ktab[:fh, :, :fn].contiguous()
            s2, a2, r2 = status[:fn].clone(), acc[:fn].clone(), rej[:fn].clone()
            res = {}
            for form in ("plain", "persistent"):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(stream):
                    c2.copy_(sub)
                    s2.zero_()
                    e0.record(stream)
                    if form == "plain":
                        for s in range(fh):
                            check(lib.mkpp_gpu_integrate_k(C.c_size_t(fn), p(c2), p(k2[s]), C.c_size_t(0), 1,
                                                           C.c_double(w.dt), C.c_double(seed), args.max_attempts, 0,
                                                           None, p(s2), p(a2), p(r2), p(ws), C.c_size_t(ws.numel()), sp),
                                  "integrate plain")
                    else:
                        check(lib.mkpp_gpu_integrate_k(C.c_size_t(fn), p(c2), p(k2), C.c_size_t(NR * fn), fh,
                                                       C.c_double(w.dt), C.c_double(seed), args.max_attempts, 1, None,
                                                       p(s2), p(a2), p(r2), p(ws), C.c_size_t(ws.numel()), sp),
                              "integrate persistent")
                    e1.record(stream)
                    stream.synchronize()
                ms = e0.elapsed_time(e1)
                res[form] = {"value": fn * fh / (ms * 1e-3), "ms": ms}
                log(f"form {form}: {ms:.0f} ms")
            result["forms"] = {"config": f"first {fn} cells x {fh} host steps", "unit": UNIT,
                               "plain": dict(res["plain"], form="one thread per cell, one launch per host step"),
                               "persistent": dict(res["persistent"], form="persistent queue + cooperative hand-off, "
                                                                         "one launch for all host steps")}

    window_adjoint = args.adjoint_window if args.adjoint_window is not None else int(w.mechanism == "ts1")
    if rank == 0 and not args.no_adjoint and window_adjoint:
        with optional_section(result, "adjoint", True):
            result["adjoint"] = adjoint_window_section(w, hs, conc0, ktab, seed, args, stream, el_ms)
            log(f"adjoint: {result['adjoint']}")
    if rank == 0 and not args.no_adjoint and not window_adjoint:
        with optional_section(result, "adjoint", True):
            # Discrete adjoint (SAPRC99 adjoint configuration): first adjoint_cells
            # cells, one 3600 s integrate() with checkpoints at accepted steps, loss
            # sum_c (O3_c - O3t_c)^2 with O3t log-normal (sigma 0.2) around the
            # forward result; gradients w.r.t. all initial concentrations and all
            # rate constants.  Reported: adjoint time / checkpointed-forward time.
            from mkpp_gb300.adjoint import Checkpoints

            cap = 1536
            # Checkpoints hold cap x NV doubles per cell: at most 100 GB of them
            # (SAPRC99: 65536 cells = 63 GB; TS1 would need 168 GB for 65536).
            na = min(n, args.adjoint_cells or 65536, int(100e9 // (cap * plan.n_var * 8)))
            ca0 = conc0[:, :na].contiguous()
            ka = ktab[0, :, :na].contiguous()
            del ktab
            torch.cuda.empty_cache()
            ck = Checkpoints(w.mechanism, na, cap, dev)
            ev_f = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev_a = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ca = ca0.clone()
            with torch.cuda.stream(stream):
                ev_f[0].record(stream)
                ck.forward(ca, ka, 3600.0, seed, args.max_attempts)
                ev_f[1].record(stream)
                stream.synchronize()
                o3 = raw["species"].index("O3")
                rng = torch.Generator(device="cpu").manual_seed(2718)
                target = ca[o3] * torch.exp(0.2 * torch.randn(na, generator=rng, dtype=f64)).to(dev)
                lam = torch.zeros_like(ca)
                lam[o3] = 2.0 * (ca[o3] - target)
                ev_a[0].record(stream)
                gc, gk = ck.adjoint(ka, lam)
                ev_a[1].record(stream)
                stream.synchronize()
            fms, ams = ev_f[0].elapsed_time(ev_f[1]), ev_a[0].elapsed_time(ev_a[1])
            cnt = ck.count.cpu().numpy()
            sts = ck.status.cpu().numpy()
            result["adjoint"] = {
                "config": f"first {na} cells, one 3600 s integrate(), loss sum (O3 - O3t)^2, O3t log-normal sigma 0.2",
                "forward_checkpointed_ms": fms, "adjoint_ms": ams, "adjoint_over_forward": ams / fms,
                "accepted_steps_pct": {q: float(np.percentile(cnt, q)) for q in (50, 99, 100)},
                "checkpoint_cap": cap, "cell_status_counts": np.bincount(sts, minlength=6).tolist(),
                "gradients": f"dL/dC0 for all species (fixed species 0) and dL/dk for all {len(raw['reactions'])} "
                             "reactions, FP64",
                "finite_gradients_frac": float(torch.isfinite(gc).all(0).double().mean()),
            }
            log(f"adjoint: forward {fms:.0f} ms, adjoint {ams:.0f} ms, ratio {ams / fms:.2f}")
            del gc, gk
            if args.tangent:
                # Forward sensitivities over the same checkpoints: a direction in
                # every initial concentration and every rate constant, scaled by
                # their values (mkpp_gpu_tangent).
                gen = torch.Generator(device="cpu").manual_seed(2719)
                dc = (ca0 * (2 * torch.rand(ca0.shape, generator=gen, dtype=f64).to(dev) - 1)).contiguous()
                dk = (ka * (2 * torch.rand(ka.shape, generator=gen, dtype=f64).to(dev) - 1)).contiguous()
                ev_t = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                with torch.cuda.stream(stream):
                    ev_t[0].record(stream)
                    tan = ck.tangent(ka, dc, dk)
                    ev_t[1].record(stream)
                    stream.synchronize()
                tms = ev_t[0].elapsed_time(ev_t[1])
                result["adjoint"].update({"tangent_ms": tms, "tangent_over_forward": tms / fms,
                                          "finite_tangent_frac": float(torch.isfinite(tan).all(0).double().mean())})
                log(f"tangent: {tms:.0f} ms, ratio {tms / fms:.2f}")
                del tan, dc, dk
            del ck
            torch.cuda.empty_cache()

    if not args.no_e2e:
        with optional_section(result, "e2e", world == 1):
            # End to end through the reference-facing host C ABI with pinned host buffers.
            host_conc = torch.from_numpy(w.conc).pin_memory()
            work_conc = host_conc.clone().pin_memory()
            host_par = [torch.from_numpy(w.param_at(s)).pin_memory() for s in range(hs)]
            t_h, r_h, p_h = (torch.from_numpy(a).pin_memory() for a in (w.temp, w.rho, w.pressure))
            rh_h = torch.from_numpy(w.rh).pin_memory()
            ctx = MechanismContext(w.mechanism, n)
            conc_np, par_np = work_conc.numpy(), [x.numpy() for x in host_par]
            ctx.set_state(conc_np, t_h.numpy(), p_h.numpy(), r_h.numpy())
            ctx.set_aerosol(relative_humidity=rh_h.numpy())
            ctx.set_cost_order(bool(args.e2e_cost_order))
            e2e_times = []
            for rep in range(1):
                work_conc.copy_(host_conc)
                barrier(world)
                t0 = time.perf_counter()
                for s in range(hs):
                    ctx.set_rate_parameters(par_np[s])
                    ctx.integrate(w.dt)
                e2e_times.append(time.perf_counter() - t0)
            e2e_s = max_over_ranks(min(e2e_times), world)
            log(f"e2e: {e2e_s:.1f} s")
            h2d = hs * n * 8 * (NS + 3 + NP)
            d2h = hs * n * 8 * NS
            if args.e2e_cost_order:
                # Every call after the first sends the cell order (int32) and
                # every call reads back the accepted and rejected counts.
                h2d += (hs - 1) * n * 4
                d2h += hs * n * 8
            result["e2e"] = {"value": cell_solves / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                             "d2h_bytes_per_step": d2h, "path": f"mkpp_set_rate_parameter_ptrs + mkpp_integrate x {hs}",
                             "cost_order": bool(args.e2e_cost_order)}
            ctx.close()

    if rank == 0 and world == 1:
        with optional_section(result, "cpu_baseline", True):
            threads = os.cpu_count() or 1
            cells = min(cpu_sample_cells(args, threads), n)
            cpu_end = []
            kind, v, el = cpu_reference_sample(w, cells, hs, threads, args.cpu_chunk, cpu_end)
            log(f"cpu baseline ({kind}): {el:.1f} s")
            # The sample's cost mix against the whole run's, from the GPU's
            # attempt counters on the same cells (the CPU solver runs the
            # same controller, so it makes the same attempts up to round-off).
            result["cpu_baseline"] = {
                "value": v, "unit": UNIT, "cores": threads, "kind": kind,
                "sample": f"first {cells} of {n} cells x {hs} host steps of {w.dt:g} s, OpenMP static chunks of "
                          f"{args.cpu_chunk} cells, OMP_PROC_BIND={os.environ.get('OMP_PROC_BIND')}, "
                          f"OMP_PLACES={os.environ.get('OMP_PLACES')}",
                "seconds": el,
                "attempts_per_cell_solve_sample": float(att[:cells].sum()) / (cells * hs),
                "attempts_per_cell_solve_run": attempts / (n * hs),
                # the timed window's end state on these cells against the CPU
                # solver's, all host steps
                "parity": parity_against(window_end[:, :cells], cpu_end[0], raw)}

    if rank == 0 and world == 1:
        with optional_section(result, "bulk", True):
            b = bulk_rate(w.mechanism, min(args.bulk_cells, n), args.bulk_attempts, stream)
            b["frac_of_fp64_peak"] = b["tflops"] / best if best else None
            result["bulk"] = b
            log(f"bulk: {b['tflops']:.3f} TFLOP/s with every lane busy")

    if rank == 0 and world == 1 and not args.no_adjoint and not window_adjoint and args.adjoint_check_cells > 0:
        with optional_section(result, "adjoint_accuracy", True):
            from mkpp_gb300.adjoint import Checkpoints

            result["adjoint_accuracy"] = adjoint_accuracy_section(
                w.mechanism, raw, plan.var_phys, solver, conc0, temp, rho, rh, params[0], seed,
                args.adjoint_check_cells, args.max_attempts, Checkpoints)
            log(f"adjoint accuracy: {result['adjoint_accuracy']}")

    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()

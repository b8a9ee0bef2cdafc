"""Attempt latency and throughput of the integrate kernels.

    python -m mkpp_gb300.coop_probe CELLS ATTEMPTS DEFER [MECHANISM]

Integrates the first CELLS cells of a mechanism's workload (first host step,
rate constants from the workload) with a bound of ATTEMPTS attempts per cell
through the persistent kernel, parking every cell after DEFER attempts
(0: never).  With DEFER = 1 each cell makes one attempt on a lane and the rest
on a whole warp; with DEFER = 0 all of them on its lane.  Few cells (one per
SM or fewer) make the time the latency of one cell's attempts; many cells
with DEFER = 0 and a small ATTEMPTS bound give the persistent kernel's
throughput with every lane busy (no tail), a case small enough for ncu.
Prints the wall time of each of two repetitions (CUDA synchronised on both
sides), the attempts made and the rate.  Used to choose
`mkpp_set_launch_tuning`'s defer_after.
"""

from __future__ import annotations

import sys
import time

import numpy as np


def main(argv=None) -> int:
    import torch

    from . import workloads
    from .api import DeviceSolver
    from .emitter.plan import flops_per_attempt, load

    argv = sys.argv[1:] if argv is None else argv
    n, cap, defer = (int(x) for x in argv[:3])
    mech = argv[3] if len(argv) > 3 else "saprc99"
    w = workloads.make(mech, n)
    s = DeviceSolver(mech)
    s.set_tuning(defer_after=defer)
    flops = flops_per_attempt(load(mech))["total"]
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    conc0 = d(w.conc)
    ktab, status = s.rate_constants(conc0, d(w.temp), d(w.rho), d(w.rh), None, d(w.param))
    for _ in range(2):
        conc = conc0.clone()
        st = status.clone()
        acc = torch.zeros(n, dtype=torch.int32, device="cuda")
        rej = torch.zeros_like(acc)
        torch.cuda.synchronize()
        t = time.time()
        s.integrate_k(conc, ktab, w.dt, max_attempts=cap, mode="persistent", status=st, accepted=acc, rejected=rej)
        torch.cuda.synchronize()
        el = time.time() - t
        att = int((acc + rej).sum())
        print(f"n={n} cap={cap} defer={defer}: {el * 1e3:.1f} ms, {att} attempts, {att / el:.3e} attempts/s, "
              f"{att * flops / el / 1e12:.3f} TFLOP/s", flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())

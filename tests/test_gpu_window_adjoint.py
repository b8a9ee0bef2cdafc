"""Gradients over several host steps with two levels of checkpoints
(mkpp_gb300.adjoint.WindowGradient).

The forward keeps only the state at each host-step boundary; the backward
recomputes one host step of one chunk of cells at a time with checkpoints at
its accepted steps and sweeps it in reverse.  Every piece is the per-call
adjoint already checked against the dense CPU adjoint and finite differences
(tests/test_gpu_adjoint.py), so the window gradient must equal, bit for bit,
the gradient autograd gives through a chain of differentiable per-host-step
solves (rosenbrock_solve, full checkpoints) with the same rate constants:
* the forward end state and the recomputed accepted steps are those of the
  persistent kernel (same controller, same arithmetic);
* dL/dC0 and dL/dk of every host step, with the cells in chunks smaller
  than the batch (so chunk boundaries are crossed).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EXTREME = {"saprc99": (11, 32, 69)}


@pytest.mark.parametrize("mech,n,hs,chunk", [("small_strato", 256, 3, 96), ("saprc99", 48, 2, 20)])
def test_window_gradient_equals_chained_solves(mech, n, hs, chunk):
    import torch

    from mkpp_gb300 import workloads
    from mkpp_gb300.adjoint import WindowGradient, rosenbrock_solve
    from mkpp_gb300.api import DeviceSolver
    from mkpp_gb300.emitter.plan import load_raw

    w = workloads.make(mech, n)
    s = DeviceSolver(mech)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    conc0 = d(w.conc)
    nr = s.sizes.reactions
    ktab = torch.empty((hs, nr, n), dtype=torch.float64, device="cuda")
    for h in range(hs):
        k, _ = s.rate_constants(conc0, d(w.temp), d(w.rho), d(w.rh), None, d(w.param_at(h)))
        for r in EXTREME.get(mech, ()):
            k[r] = torch.clamp(k[r], max=1e3)
        ktab[h].copy_(k)
    seed = s.default_seed
    o3 = load_raw(mech)["species"].index("O3")
    target = conc0[o3] * 0.9

    wg = WindowGradient(mech, n, hs, conc0.device, cap=2048, chunk=chunk)
    end = wg.forward(conc0.clone(), ktab, w.dt, seed)
    lam = torch.zeros_like(end)
    lam[o3] = 2.0 * (end[o3] - target)
    gc, gk = wg.backward(ktab, lam)
    torch.cuda.synchronize()
    ok = (wg.status == 0) & (wg.forward_status == 0) & torch.isfinite(end).all(0)
    assert ok.float().mean() > 0.9

    # The same gradient through autograd over chained per-host-step solves.
    c = conc0.clone().requires_grad_(True)
    ks = [ktab[h].clone().requires_grad_(True) for h in range(hs)]
    x = c
    for h in range(hs):
        x = rosenbrock_solve(x, ks[h], mech, dt=w.dt, cap=2048, seed=seed)
    loss = ((x[o3] - target)[ok] ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()

    assert torch.equal(end[:, ok], x.detach()[:, ok])
    assert torch.equal(gc[:, ok], c.grad[:, ok])
    for h in range(hs):
        assert torch.equal(gk[h][:, ok], ks[h].grad[:, ok]), f"host step {h}"

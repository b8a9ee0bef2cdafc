"""Discrete adjoint on the GPU (mkpp_gpu_integrate_checkpoint / mkpp_gpu_adjoint).

Checks, with the accepted-step sequence of the checkpointed forward frozen:
* against a dense FP64 CPU discrete adjoint (oracle/adjoint_ref.py) of the same
  steps: gradients w.r.t. the initial state and the rate constants agree to
  1e-8 of the cell's largest |x * dL/dx| (scale-free sensitivities), or to
  8x the cell's round-off floor where that is larger.  The floor is how far
  the dense adjoint itself moves when k and y0 are perturbed by one ulp: up
  to 3e-8 on stiff SAPRC99 cells (seeded case), 1e-12 on others;
* against central finite differences (h = 1e-6 relative) of the loss
  L = sum_c (O3_c(dt) - target_c)^2 through the GPU replay of the same steps;
* the torch.autograd.Function returns those gradients and the same forward
  result as the plain integrate kernel.
SAPRC99 runs with its three 1e33-1e37 1/s rate constants moderated to 1e3
(see test_gpu_parity.EXTREME_RATES): with them the problem is too
ill-conditioned for differences at 1e-6 to mean anything.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EXTREME = {"saprc99": (11, 32, 69)}
DT = {"chapman": 300.0, "small_strato": 300.0, "saprc99": 300.0}


def _case(mech, n):
    import torch

    from mkpp_gb300 import workloads
    from mkpp_gb300.adjoint import Checkpoints
    from mkpp_gb300.api import DeviceSolver

    w = workloads.make(mech, n)
    s = DeviceSolver(mech)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    conc0 = d(w.conc)
    ktab, st = s.rate_constants(conc0, d(w.temp), d(w.rho), d(w.rh), None, d(w.param))
    for r in EXTREME.get(mech, ()):
        ktab[r] = torch.clamp(ktab[r], max=1e3)
    ck = Checkpoints(mech, n, 2048, conc0.device)
    conc = conc0.clone()
    ck.forward(conc, ktab, DT[mech], s.default_seed)
    torch.cuda.synchronize()
    return w, s, conc0, conc, ktab, ck


def _roundoff_floor(dm, y0, k, hs, lam, g0, gk0, trials=2):
    """Largest relative change of the dense adjoint under one-ulp perturbations
    of k and y0 (same step sequence): the agreement two correct FP64
    implementations can be expected to reach on this cell."""
    rng = np.random.default_rng(11)
    sy = max(np.abs(g0 * y0).max(), 1e-300)
    sk = max(np.abs(gk0 * k).max(), 1e-300)
    fy = fk = 0.0
    for _ in range(trials):
        kp = k * (1.0 + rng.integers(-1, 2, size=k.size) * 2.0**-52)
        yp = y0 * (1.0 + rng.integers(-1, 2, size=y0.size) * 2.0**-52)
        _, tape = dm.forward(yp, kp, hs)
        g1, gk1 = dm.adjoint(kp, tape, lam)
        fy = max(fy, np.abs((g1 - g0) * y0).max() / sy)
        fk = max(fk, np.abs((gk1 - gk0) * k).max() / sk)
    return fy, fk


@pytest.mark.parametrize("mech", ["chapman", "small_strato", "saprc99"])
def test_adjoint_matches_dense_cpu_adjoint(built_libs, mech):
    import torch

    from oracle.adjoint_ref import DenseModel

    n = 4
    w, s, conc0, conc, ktab, ck = _case(mech, n)
    assert int(ck.status.sum()) == 0
    dm = DenseModel(mech)
    vp = dm.p.var_phys
    yT = conc.cpu().numpy()
    lam = np.zeros_like(yT)
    lam[vp] = 1.0 / np.maximum(np.abs(yT[vp]), 1.0)
    gc, gk = ck.adjoint(ktab, torch.from_numpy(lam).cuda())
    torch.cuda.synchronize()
    gc, gk = gc.cpu().numpy(), gk.cpu().numpy()
    cnt = ck.count.cpu().numpy()
    hs_all = ck.h.cpu().numpy()
    k = ktab.cpu().numpy()
    for c in range(n):
        y0 = w.conc[vp, c]
        yT_cpu, tape = dm.forward(y0, k[:, c], hs_all[: cnt[c], c])
        np.testing.assert_allclose(yT_cpu, yT[vp, c], rtol=1e-9, atol=1e-6)
        g0, gkc = dm.adjoint(k[:, c], tape, lam[vp, c])
        scale = max(np.abs(g0 * y0).max(), 1e-300)
        sk = max(np.abs(gkc * k[:, c]).max(), 1e-300)
        floor_y, floor_k = _roundoff_floor(dm, y0, k[:, c], hs_all[: cnt[c], c], lam[vp, c], g0, gkc)
        assert np.max(np.abs((gc[vp, c] - g0) * y0)) <= max(1e-8, 8 * floor_y) * scale
        assert np.max(np.abs((gk[:, c] - gkc) * k[:, c])) <= max(1e-8, 8 * floor_k) * sk


@pytest.mark.parametrize("mech", ["small_strato", "saprc99"])
def test_adjoint_matches_central_differences(built_libs, mech):
    import torch

    n = 64
    w, s, conc0, conc, ktab, ck = _case(mech, n)
    ok = (ck.status == 0).cpu().numpy()
    from mkpp_gb300.emitter.plan import load, load_raw

    o3 = load_raw(mech)["species"].index("O3")
    target = (conc[o3] * 1.1).clone()

    def loss(cend):
        return ((cend[o3] - target) ** 2)

    lam = torch.zeros_like(conc)
    lam[o3] = 2.0 * (conc[o3] - target)
    gc, gk = ck.adjoint(ktab, lam)
    torch.cuda.synchronize()
    vp = load(mech).var_phys
    rng = np.random.default_rng(5)
    species = [o3] + list(rng.choice(vp, size=4, replace=False))
    for sp in species:
        for sign_delta in (1e-6,):
            d = sign_delta * conc0[sp].abs()
            cp = conc0.clone(); cp[sp] += d
            cm = conc0.clone(); cm[sp] -= d
            ck.replay(cp, ktab)
            ck.replay(cm, ktab)
            torch.cuda.synchronize()
            fd = ((loss(cp) - loss(cm)) / (2 * d)).cpu().numpy()
            ad = gc[sp].cpu().numpy()
            scale = (loss(conc).cpu().numpy() + 1e-300)
            # compare relative sensitivities C0 * dL/dC0 against the loss size
            c0 = conc0[sp].cpu().numpy()
            err = np.abs((fd - ad) * c0) / scale
            assert np.median(err[ok]) <= 1e-5, (sp, np.median(err[ok]))
            assert np.percentile(err[ok], 90) <= 1e-3, (sp, np.percentile(err[ok], 90))
    for r in list(rng.choice(ktab.shape[0], size=4, replace=False)):
        d = 1e-6 * ktab[r].abs()
        if float(d.max()) == 0.0:
            continue
        kp = ktab.clone(); kp[r] += d
        km = ktab.clone(); km[r] -= d
        cp, cm = conc0.clone(), conc0.clone()
        ck.replay(cp, kp)
        ck.replay(cm, km)
        torch.cuda.synchronize()
        fd = ((loss(cp) - loss(cm)) / (2 * d.clamp(min=1e-300))).cpu().numpy()
        ad = gk[r].cpu().numpy()
        kk = ktab[r].cpu().numpy()
        err = np.abs((fd - ad) * kk) / (loss(conc).cpu().numpy() + 1e-300)
        live = ok & (kk > 0)
        if live.any():
            assert np.median(err[live]) <= 1e-5, (r, np.median(err[live]))


def test_autograd_function(built_libs):
    import torch

    from mkpp_gb300 import workloads
    from mkpp_gb300.adjoint import rosenbrock_solve
    from mkpp_gb300.api import DeviceSolver

    mech = "small_strato"
    w = workloads.make(mech, 128)
    s = DeviceSolver(mech)
    conc0 = torch.from_numpy(w.conc).cuda().requires_grad_(True)
    ktab, _ = s.rate_constants(conc0.detach(), param=torch.from_numpy(w.param).cuda())
    ktab = ktab.clone().requires_grad_(True)
    cend = rosenbrock_solve(conc0, ktab, mech, dt=300.0)
    # same forward result as the plain integrate kernel
    ref = conc0.detach().clone()
    s.integrate_k(ref, ktab.detach(), 300.0, mode="plain")
    torch.cuda.synchronize()
    assert torch.equal(cend.detach(), ref)
    loss = (cend[2] ** 2).sum()
    loss.backward()
    assert conc0.grad is not None and ktab.grad is not None
    assert torch.isfinite(conc0.grad).all() and torch.isfinite(ktab.grad).all()
    assert float(conc0.grad.abs().sum()) > 0.0

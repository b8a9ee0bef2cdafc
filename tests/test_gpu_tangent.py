"""Tangent (forward sensitivities) on the GPU: mkpp_gpu_tangent and the
forward-mode rule of the autograd function.

On the accepted-step sequence of a checkpointed forward (DT = 300 s, four
seeded cells per mechanism):
* the GPU tangent against the emitted tangent compiled for the host
  (tests/hostsim_lib.py), stepped through the GPU's own checkpoints.  Both
  run the same emitted operations (explicit fma, IEEE division), so they are
  expected to agree bit for bit; the bound is 1e-12 of the cell's largest
  |dC|.  The host forward also reproduces every next checkpoint from the
  previous one to the same bound;
* the transpose identity with the GPU adjoint, per cell:
  <T (dC0, dk), lam> = <dC0, dL/dC0> + <dk, dL/dk> with L = <lam, C_end>, to
  1e-10 of the sum of the absolute terms (measured on the CPU over the same
  trajectories: at most 5e-13).  The reference's own tests check the same
  identity for its frozen-Jacobian pair (test_adjoint_identity.py);
* forward-mode autograd (torch.autograd.forward_ad) through rosenbrock_solve
  returns the kernel's tangent and passes the fixed species through.
SAPRC99 runs with its three 1e33-1e37 1/s rate constants moderated to 1e3, as
in the adjoint tests.
"""
import numpy as np
import pytest

import hostsim_lib

pytestmark = pytest.mark.gpu

EXTREME = {"saprc99": (11, 32, 69)}
MECHS = ["chapman", "small_strato", "saprc99"]
DT = 300.0
CELLS = 4


def _case(mech):
    import torch

    from mkpp_gb300 import workloads
    from mkpp_gb300.adjoint import Checkpoints
    from mkpp_gb300.api import DeviceSolver

    w = workloads.make(mech, CELLS)
    s = DeviceSolver(mech)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    conc0 = d(w.conc)
    ktab, _ = s.rate_constants(conc0, d(w.temp), d(w.rho), d(w.rh), None, d(w.param))
    for r in EXTREME.get(mech, ()):
        ktab[r] = torch.clamp(ktab[r], max=1e3)
    ck = Checkpoints(mech, CELLS, 2048, conc0.device)
    conc = conc0.clone()
    ck.forward(conc, ktab, DT, s.default_seed)
    torch.cuda.synchronize()
    assert int(ck.status.sum()) == 0
    return s, conc0, conc, ktab, ck


def _directions(conc0, ktab, seed=3):
    import torch

    rng = np.random.default_rng(seed)
    c, k = conc0.cpu().numpy(), ktab.cpu().numpy()
    dc = rng.uniform(-1.0, 1.0, c.shape) * np.abs(c)
    dk = rng.uniform(-1.0, 1.0, k.shape) * k
    return torch.from_numpy(dc).cuda(), torch.from_numpy(dk).cuda()


@pytest.mark.parametrize("mech", MECHS)
def test_tangent_matches_host_program(built_libs, mech, tmp_path):
    import torch

    from mkpp_gb300.emitter.plan import load

    s, conc0, conc, ktab, ck = _case(mech)
    dc, dk = _directions(conc0, ktab)
    out = ck.tangent(ktab, dc, dk)
    torch.cuda.synchronize()
    out = out.cpu().numpy()
    vp = load(mech).var_phys
    fixed = np.setdiff1d(np.arange(out.shape[0]), vp)
    assert (out[fixed] == 0.0).all()
    lib = hostsim_lib.compile(tmp_path, mech)
    ys, hs, ns = ck.y.cpu().numpy(), ck.h.cpu().numpy(), ck.count.cpu().numpy()
    k, dcn, dkn = ktab.cpu().numpy(), dc.cpu().numpy(), dk.cpu().numpy()
    for c in range(CELLS):
        assert ns[c] > 0
        dy = dcn[vp, c]
        for st in range(ns[c]):
            y = ys[st, :, c]
            dy, y_new, status = hostsim_lib.tangent_step(lib, y, k[:, c], hs[st, c], dy, dkn[:, c])
            assert status == 0
            nxt = ys[st + 1, :, c] if st + 1 < ns[c] else conc.cpu().numpy()[vp, c]
            assert np.abs(y_new - nxt).max() <= 1e-12 * np.abs(nxt).max()
        assert np.abs(out[vp, c] - dy).max() <= 1e-12 * np.abs(dy).max(), (c, ns[c])


@pytest.mark.parametrize("mech", MECHS)
def test_tangent_is_the_transpose_of_the_adjoint(built_libs, mech):
    import torch

    s, conc0, conc, ktab, ck = _case(mech)
    dc, dk = _directions(conc0, ktab)
    rng = np.random.default_rng(7)
    ce = conc.cpu().numpy()
    lam = torch.from_numpy(rng.uniform(-1.0, 1.0, ce.shape) / np.maximum(np.abs(ce), 1.0)).cuda()
    t = ck.tangent(ktab, dc, dk)
    gc, gk = ck.adjoint(ktab, lam)
    torch.cuda.synchronize()
    t, gc, gk, lam = (x.cpu().numpy() for x in (t, gc, gk, lam))
    dc, dk = dc.cpu().numpy(), dk.cpu().numpy()
    lhs = (t * lam).sum(axis=0)
    rhs = (dc * gc).sum(axis=0) + (dk * gk).sum(axis=0)
    scale = np.abs(t * lam).sum(axis=0) + np.abs(dc * gc).sum(axis=0) + np.abs(dk * gk).sum(axis=0)
    assert (scale > 0).all()
    assert (np.abs(lhs - rhs) <= 1e-10 * scale).all(), np.abs(lhs - rhs) / scale


def test_forward_mode_autograd(built_libs):
    import torch
    import torch.autograd.forward_ad as fwAD

    from mkpp_gb300.adjoint import rosenbrock_solve
    from mkpp_gb300.emitter.plan import load

    mech = "small_strato"
    s, conc0, conc, ktab, ck = _case(mech)
    dc, dk = _directions(conc0, ktab)
    with fwAD.dual_level():
        out = rosenbrock_solve(fwAD.make_dual(conc0, dc), fwAD.make_dual(ktab, dk), mech, dt=DT)
        primal, tangent = fwAD.unpack_dual(out)
        primal, tangent = primal.clone(), tangent.clone()
    ref = ck.tangent(ktab, dc, dk)
    torch.cuda.synchronize()
    assert torch.equal(primal, conc)
    vp = torch.tensor(load(mech).var_phys, device=conc.device)
    assert torch.equal(tangent[vp], ref[vp])
    fixed = torch.tensor(np.setdiff1d(np.arange(conc.shape[0]), load(mech).var_phys), device=conc.device)
    assert torch.equal(tangent[fixed], dc[fixed])

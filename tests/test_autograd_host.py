"""Host logic of the differentiable solve (mkpp_gb300/adjoint.py), on the CPU.

The GPU checkpoint object is replaced by a linear stand-in with the C
entries' conventions (variable species only; fixed species 0 in
mkpp_gpu_adjoint's and mkpp_gpu_tangent's outputs):
conc_end[var] = 2 conc0[var] + sum_r k_r, conc_end[fixed] = conc0[fixed].
Checks that the autograd function passes the fixed species through in both
directions, and that forward mode and reverse mode give the same derivative.
"""
import numpy as np
import pytest
import torch

from mkpp_gb300 import adjoint as adj
from mkpp_gb300.emitter.plan import load, load_raw

MECH = "small_strato"


class _LinearCheckpoints:
    def __init__(self, mechanism, ncells, cap, device):
        raw = load_raw(mechanism)
        self.n = ncells
        self.vp = torch.tensor(load(mechanism).var_phys)
        self.sizes = type("S", (), {"species": len(raw["species"]), "reactions": len(raw["reactions"])})

    def forward(self, conc, ktab, dt, seed, max_attempts=20000):
        conc[self.vp] = 2.0 * conc[self.vp] + ktab.sum(0)

    def tangent(self, ktab, dconc0, dk=None):
        out = torch.zeros((self.sizes.species, self.n), dtype=torch.float64)
        out[self.vp] = 2.0 * dconc0[self.vp] + (0.0 if dk is None else dk.sum(0))
        return out

    def adjoint(self, ktab, lam):
        gc = torch.zeros((self.sizes.species, self.n), dtype=torch.float64)
        gc[self.vp] = 2.0 * lam[self.vp]
        gk = lam[self.vp].sum(0).expand(self.sizes.reactions, self.n).clone()
        return gc, gk


@pytest.fixture
def linear(monkeypatch):
    monkeypatch.setattr(adj, "Checkpoints", _LinearCheckpoints)
    raw = load_raw(MECH)
    rng = np.random.default_rng(2)
    ns, nr, n = len(raw["species"]), len(raw["reactions"]), 5
    t = lambda *s: torch.from_numpy(rng.uniform(0.5, 1.5, s))  # noqa: E731
    fixed = [i for i, f in enumerate(raw["fixed"]) if f]
    assert fixed, "the case needs a mechanism with fixed species"
    return t(ns, n), t(nr, n), t(ns, n), t(nr, n), t(ns, n), torch.tensor(load(MECH).var_phys), torch.tensor(fixed)


def test_reverse_mode_passes_fixed_species_through(linear):
    c0, k, _, _, w, vp, fixed = linear
    c0.requires_grad_(True)
    k.requires_grad_(True)
    out = adj.rosenbrock_solve(c0, k, MECH, dt=1.0, seed=1e-6)
    assert torch.equal(out[fixed], c0.detach()[fixed])
    (out * w).sum().backward()
    assert torch.equal(c0.grad[vp], 2.0 * w[vp])
    assert torch.equal(c0.grad[fixed], w[fixed])
    assert torch.allclose(k.grad, w[vp].sum(0).expand_as(k))


def test_forward_mode_matches_reverse_mode(linear):
    import torch.autograd.forward_ad as fwAD

    c0, k, dc, dk, w, vp, fixed = linear
    with fwAD.dual_level():
        out = adj.rosenbrock_solve(fwAD.make_dual(c0, dc), fwAD.make_dual(k, dk), MECH, dt=1.0, seed=1e-6)
        _, tan = fwAD.unpack_dual(out)
        tan = tan.clone()
    assert torch.equal(tan[vp], 2.0 * dc[vp] + dk.sum(0))
    assert torch.equal(tan[fixed], dc[fixed])
    c0r, kr = c0.clone().requires_grad_(True), k.clone().requires_grad_(True)
    (adj.rosenbrock_solve(c0r, kr, MECH, dt=1.0, seed=1e-6) * w).sum().backward()
    lhs = (tan * w).sum()
    rhs = (dc * c0r.grad).sum() + (dk * kr.grad).sum()
    assert torch.allclose(lhs, rhs, rtol=1e-14, atol=0)


def test_forward_mode_without_rate_tangent(linear):
    import torch.autograd.forward_ad as fwAD

    c0, k, dc, _, _, vp, fixed = linear
    with fwAD.dual_level():
        out = adj.rosenbrock_solve(fwAD.make_dual(c0, dc), k, MECH, dt=1.0, seed=1e-6)
        tan = fwAD.unpack_dual(out).tangent.clone()
    assert torch.equal(tan[vp], 2.0 * dc[vp])
    assert torch.equal(tan[fixed], dc[fixed])

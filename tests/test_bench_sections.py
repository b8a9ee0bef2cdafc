"""Host logic of bench.py's secondary sections, on the CPU with stand-ins for
the GPU entries: the adjoint's accuracy check (central differences through
the recorded steps), the L2 rule of the timed loop and the workload
description."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

torch = pytest.importorskip("torch")


class _Solver:
    """rate_constants of a two-reaction stand-in: k depends on the state."""

    def rate_constants(self, conc, temp, rho, rh, clw, param):
        k = torch.stack([1e-3 * (1.0 + temp / 300.0), 2e-4 * (1.0 + rho * 0.0 + param[0])])
        return k, torch.zeros(conc.shape[1], dtype=torch.int32)


class _Checkpoints:
    """A smooth per-cell map in place of the solver: y_end = y0 exp(-(k0 +
    k1) t) + k0 t on the variable rows, fixed rows unchanged; replay is the
    same map, adjoint its exact transpose."""

    T = 3.0

    def __init__(self, mechanism, n, cap, dev, var_rows=(0, 1, 2)):
        self.var = list(var_rows)

    def _map(self, c, k):
        e = torch.exp(-(k[0] + k[1]) * self.T)
        c[self.var] = c[self.var] * e + k[0] * self.T

    def forward(self, c, k, dt, seed, max_attempts):
        self.c0 = c.clone()
        self.status = torch.zeros(c.shape[1], dtype=torch.int32)
        self._map(c, k)

    def replay(self, c, k):
        self._map(c, k)

    def adjoint(self, k, lam):
        e = torch.exp(-(k[0] + k[1]) * self.T)
        gc = torch.zeros_like(lam)
        gc[self.var] = lam[self.var] * e
        dy_dsum = -self.T * self.c0[self.var] * e          # d y_end / d(k0 + k1)
        s = (lam[self.var] * dy_dsum).sum(0)
        gk = torch.stack([s + self.T * lam[self.var].sum(0), s])
        return gc, gk


def test_adjoint_accuracy_section_matches_an_exact_adjoint():
    import bench

    n, ns = 64, 4
    gen = torch.Generator().manual_seed(1)
    conc0 = torch.rand((ns, n), generator=gen, dtype=torch.float64) + 0.5
    temp = torch.full((n,), 290.0, dtype=torch.float64)
    rho = torch.full((n,), 2.4e19, dtype=torch.float64)
    rh = torch.full((n,), 0.5, dtype=torch.float64)
    param = torch.rand((1, n), generator=gen, dtype=torch.float64)
    raw = {"species": ["O3", "NO", "NO2", "M"]}
    out = bench.adjoint_accuracy_section("stand-in", raw, [0, 1, 2], _Solver(), conc0, temp, rho, rh, param,
                                         1e-6, 32, 20000, _Checkpoints)
    assert out["cells_status_ok"] == 32
    for part in ("initial_concentrations", "rate_constants"):
        st = out[part]
        assert st["cells"] == 32
        assert st["max_rel_error"] < 1e-6, (part, st)
        assert st["frac_within_1e-4"] == 1.0 and st["frac_consistent"] == 1.0
        assert st["median_difference_noise"] < 1e-6


def test_adjoint_accuracy_section_sees_a_wrong_gradient():
    """A planted error in the stand-in's adjoint shows up in the statistics."""
    import bench

    class Wrong(_Checkpoints):
        def adjoint(self, k, lam):
            gc, gk = super().adjoint(k, lam)
            return gc * 1.01, gk

    n = 16
    conc0 = torch.full((4, n), 1.0, dtype=torch.float64)
    one = torch.ones(n, dtype=torch.float64)
    out = bench.adjoint_accuracy_section("stand-in", {"species": ["O3", "NO", "NO2", "M"]}, [0, 1, 2], _Solver(),
                                         conc0, 290.0 * one, one, one, torch.zeros((1, n), dtype=torch.float64),
                                         1e-6, n, 20000, Wrong)
    assert out["initial_concentrations"]["median_rel_error"] > 5e-3
    assert out["initial_concentrations"]["frac_consistent"] == 0.0
    assert out["rate_constants"]["max_rel_error"] < 1e-6


@pytest.mark.parametrize("name,cells,fits", [("chapman", 4096, True), ("small_strato", 65536, True),
                                             ("saprc99", 262144, False)])
def test_l2_rule_of_the_timed_loop(name, cells, fits):
    """Inputs that fit in L2 (small configurations) are flushed before every
    timed step; SAPRC99's window inputs are far larger than L2."""
    import bench
    from mkpp_gb300 import workloads

    w = workloads.make(name, 256)
    hs = w.host_steps
    per_cell = bench.window_input_bytes(w, hs) / 256
    big = per_cell * cells > 2 * bench.L2_BYTES
    assert big == (not fits)
    assert bench.L2_FLUSH_BYTES > bench.L2_BYTES


def test_workload_description_names_the_tableau():
    import bench
    from mkpp_gb300 import workloads

    for name, tab in (("chapman", "ROS-3"), ("chapman_rodas3", "RODAS-3")):
        w = workloads.make(name, 128)
        cfg = bench.workload_config(w, w.host_steps)
        assert cfg["tableau"] == tab and f", {tab}, " in cfg["workload"]
        assert "flushed" in cfg["l2"]

"""Differentiable Rosenbrock solve: torch.autograd.Function over the GPU
checkpointed forward, discrete-adjoint and tangent kernels.

    conc_end = rosenbrock_solve(conc0, ktab, "saprc99", dt=3600.0)
    loss = ((conc_end[o3] - target) ** 2).sum()
    loss.backward()          # conc0.grad: dL/dC0, ktab.grad: dL/dk

conc0 is (species, cells) and ktab (reactions, cells), float64 CUDA tensors
(LayoutLeft, cell index innermost).  The forward records the state and step
size of every accepted step; the backward sweeps them in reverse
(``mkpp_gpu_adjoint``), recomputing each step's stages, and returns the exact
gradient of the computed solution for that step sequence (the step sizes are
treated as constants, as in any discrete adjoint of an adaptive method).

Forward mode (``torch.autograd.forward_ad`` dual tensors) sweeps the same
steps first to last (``mkpp_gpu_tangent``) and returns the directional
derivative d conc_end (d conc0, d ktab), the transpose of the backward.

integrate() leaves the fixed species as they are, so conc_end's fixed rows
are conc0's: both directions pass those rows through unchanged.  Fixed
species act on the variable ones only through ktab.
"""

from __future__ import annotations

import ctypes as C

import torch

from .api import MKPP_SUCCESS, MkppError, load_library, sizes
from .emitter.plan import load_raw


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class Checkpoints:
    """Device buffers of one checkpointed forward."""

    def __init__(self, mechanism: str, ncells: int, cap: int, device):
        self.lib = load_library(mechanism)
        self.sizes = sizes(mechanism)
        self.n = ncells
        self.cap = cap
        nv = self.sizes.variable
        self.y = torch.empty((cap, nv, ncells), dtype=torch.float64, device=device)
        self.h = torch.empty((cap, ncells), dtype=torch.float64, device=device)
        self.count = torch.zeros(ncells, dtype=torch.int32, device=device)
        ws = int(self.lib.mkpp_gpu_adjoint_workspace_bytes(C.c_size_t(ncells)))
        self.ws = torch.zeros(ws + 256, dtype=torch.uint8, device=device)
        self.tws = None  # the tangent's workspace, allocated on first use

    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def forward(self, conc, ktab, dt, seed, max_attempts=20000):
        n = self.n
        dev = conc.device
        self.status = torch.zeros(n, dtype=torch.int32, device=dev)
        self.acc = torch.zeros(n, dtype=torch.int32, device=dev)
        self.rej = torch.zeros(n, dtype=torch.int32, device=dev)
        rc = self.lib.mkpp_gpu_integrate_checkpoint(
            C.c_size_t(n), _p(conc), _p(ktab), C.c_double(dt), C.c_double(seed), C.c_int(max_attempts),
            C.c_int(self.cap), _p(self.y), _p(self.h), _p(self.count), _p(self.status), _p(self.acc),
            _p(self.rej), _p(self.ws), C.c_size_t(self.ws.numel()), self._stream())
        if rc != MKPP_SUCCESS:
            raise MkppError(rc)

    def replay(self, conc, ktab):
        rc = self.lib.mkpp_gpu_integrate_replay(
            C.c_size_t(self.n), _p(conc), _p(ktab), C.c_int(self.cap), _p(self.h), _p(self.count), _p(self.ws),
            C.c_size_t(self.ws.numel()), self._stream())
        if rc != MKPP_SUCCESS:
            raise MkppError(rc)

    def tangent(self, ktab, dconc0, dk=None):
        """d conc_end applied to (dconc0, dk) for the recorded steps (fixed
        species 0)."""
        if self.tws is None:
            ws = int(self.lib.mkpp_gpu_tangent_workspace_bytes(C.c_size_t(self.n)))
            self.tws = torch.zeros(ws + 256, dtype=torch.uint8, device=dconc0.device)
        out = torch.empty((self.sizes.species, self.n), dtype=torch.float64, device=dconc0.device)
        rc = self.lib.mkpp_gpu_tangent(
            C.c_size_t(self.n), _p(ktab), C.c_int(self.cap), _p(self.y), _p(self.h), _p(self.count),
            _p(dconc0), _p(dk), _p(out), _p(self.tws), C.c_size_t(self.tws.numel()), self._stream())
        if rc != MKPP_SUCCESS:
            raise MkppError(rc)
        return out

    def adjoint(self, ktab, lam_end):
        gc = torch.empty((self.sizes.species, self.n), dtype=torch.float64, device=lam_end.device)
        gk = torch.empty((self.sizes.reactions, self.n), dtype=torch.float64, device=lam_end.device)
        rc = self.lib.mkpp_gpu_adjoint(
            C.c_size_t(self.n), _p(ktab), C.c_int(self.cap), _p(self.y), _p(self.h), _p(self.count),
            _p(lam_end), _p(gc), _p(gk), _p(self.ws), C.c_size_t(self.ws.numel()), self._stream())
        if rc != MKPP_SUCCESS:
            raise MkppError(rc)
        return gc, gk


class RosenbrockSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, conc0, ktab, mechanism, dt, cap, seed, max_attempts):
        conc = conc0.detach().clone().contiguous()
        k = ktab.detach().contiguous()
        ck = Checkpoints(mechanism, conc.shape[1], cap, conc.device)
        ck.forward(conc, k, dt, seed, max_attempts)
        ctx.ck = ck
        ctx.k = k
        ctx.fixed = _fixed_rows(mechanism, conc.device)
        ctx.save_for_backward(k)
        return conc

    @staticmethod
    def backward(ctx, grad_out):
        (k,) = ctx.saved_tensors
        g = grad_out.contiguous()
        gc, gk = ctx.ck.adjoint(k, g)
        gc[ctx.fixed] = g[ctx.fixed]
        return gc, gk, None, None, None, None, None

    @staticmethod
    def jvp(ctx, dconc0, dktab, *_):
        k = ctx.k
        if dconc0 is None:
            dconc0 = torch.zeros((ctx.ck.sizes.species, ctx.ck.n), dtype=torch.float64, device=k.device)
        d = dconc0.contiguous()
        out = ctx.ck.tangent(k, d, None if dktab is None else dktab.contiguous())
        out[ctx.fixed] = d[ctx.fixed]
        return out


class WindowGradient:
    """Gradient of a loss on the state after several host steps (one
    integrate() call per host step, each with its own rate constants), with
    two levels of checkpoints so that memory stays bounded at any cell count:

    * level 1, in the forward: the state at every host-step boundary
      ((host_steps + 1) x species x cells doubles), the integration itself
      one persistent launch per host step;
    * level 2, in the backward, host steps last to first and cells in chunks
      of ``chunk``: the accepted steps of the chunk's host step are recomputed
      from its level-1 state (mkpp_gpu_integrate_checkpoint, the same
      controller and arithmetic, so the same steps and states as the forward)
      and swept in reverse (mkpp_gpu_adjoint), which turns lambda at the end
      of the host step into lambda at its start and gives dL/dk of that host
      step.

    Checkpoint memory is chunk x cap x variable species doubles, whatever the
    cell count.  A cell whose host step needs more than ``cap`` accepted steps
    ends with status 5 in ``status`` and non-finite gradients."""

    def __init__(self, mechanism: str, ncells: int, host_steps: int, device, cap: int = 768,
                 chunk: int = 65536):
        self.mechanism = mechanism
        self.lib = load_library(mechanism)
        self.sizes = sizes(mechanism)
        self.n = ncells
        self.hs = host_steps
        self.cap = cap
        self.chunk = min(chunk, ncells)
        self.device = device
        self.bounds = torch.empty((host_steps + 1, self.sizes.species, ncells), dtype=torch.float64, device=device)
        self.fixed = _fixed_rows(mechanism, device)
        self.status = torch.zeros(ncells, dtype=torch.int32, device=device)

    def forward(self, conc, ktab, dt, seed, max_attempts=20000, solver=None):
        """Integrates conc in place over the host steps (ktab [host step]
        [reaction][cell]), keeping every boundary state."""
        from .api import DeviceSolver

        s = solver or DeviceSolver(self.mechanism)
        self.dt, self.seed, self.max_attempts = dt, seed, max_attempts
        self.bounds[0].copy_(conc)
        st = torch.zeros(self.n, dtype=torch.int32, device=conc.device)
        for h in range(self.hs):
            s.integrate_k(conc, ktab[h], dt, seed=seed, max_attempts=max_attempts, status=st)
            self.bounds[h + 1].copy_(conc)
        self.forward_status = st
        return conc

    def backward(self, ktab, lam_end):
        """(dL/dconc0 [species][cell], dL/dk [host step][reaction][cell])
        from lam_end = dL/dconc_end.  Fixed species pass their lambda through
        (integrate() leaves them unchanged; they act through ktab)."""
        n, c = self.n, self.chunk
        lam = lam_end.detach().clone().contiguous()
        gk = torch.empty((self.hs, self.sizes.reactions, n), dtype=torch.float64, device=lam.device)
        ck = Checkpoints(self.mechanism, c, self.cap, lam.device)
        self.status.zero_()
        for h in reversed(range(self.hs)):
            for c0 in range(0, n, c):
                c1 = min(c0 + c, n)
                if c1 - c0 != ck.n:
                    ck = Checkpoints(self.mechanism, c1 - c0, self.cap, lam.device)
                y = self.bounds[h][:, c0:c1].contiguous()
                k = ktab[h][:, c0:c1].contiguous()
                ck.forward(y, k, self.dt, self.seed, self.max_attempts)
                lam_c = lam[:, c0:c1].contiguous()
                gc, gkc = ck.adjoint(k, lam_c)
                gc[self.fixed] = lam_c[self.fixed]
                lam[:, c0:c1] = gc
                gk[h][:, c0:c1] = gkc
                bad = ck.status != 0
                self.status[c0:c1] = torch.where((self.status[c0:c1] == 0) & bad, ck.status, self.status[c0:c1])
        return lam, gk


def _fixed_rows(mechanism: str, device):
    """Indices of the fixed species in the (species, cells) layout."""
    fixed = load_raw(mechanism)["fixed"]
    return torch.tensor([i for i, f in enumerate(fixed) if f], dtype=torch.long, device=device)


def rosenbrock_solve(conc0, ktab, mechanism: str, dt: float, cap: int = 1280, seed: float | None = None,
                     max_attempts: int = 20000):
    """One integrate() call over dt, differentiable w.r.t. conc0 and ktab."""
    if seed is None:
        seed = float(load_raw(mechanism)["initial_step_seed"])
    return RosenbrockSolve.apply(conc0, ktab, mechanism, dt, cap, seed, max_attempts)

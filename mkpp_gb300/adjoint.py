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

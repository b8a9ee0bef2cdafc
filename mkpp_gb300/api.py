"""Python host interface of the GB300 MKPP solver libraries.

Two layers, both thin ctypes bindings over the C ABI in ``include/mkpp.h``:

* :class:`MechanismContext` mirrors the reference's C++ host wrapper
  (``src/mkpp/templates/host_api/mkpp.hpp.j2:28-152``): a handle over
  caller-owned host arrays, ``integrate(dt)`` in place, ``evaluate_rates`` and
  ``evaluate_jacobian``, errors raised with the handle's last error message.
* :class:`DeviceSolver` drives the ``mkpp_gpu_*`` device entry points on torch
  CUDA tensors and the current torch stream, for callers that keep their
  state resident on the GPU.

Arrays are LayoutLeft with the cell index innermost: a (species, cells)
C-contiguous array is exactly ``conc[cell + num_cells * species]``.
There is no CPU fallback: a missing library raises.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

LIB_DIR = Path(__file__).resolve().parent / "lib"

MKPP_SUCCESS = 0
ERRORS = {
    -101: "MKPP_ERROR_NULL_POINTER",
    -102: "MKPP_ERROR_INVALID_HANDLE",
    -103: "MKPP_ERROR_INVALID_ARGUMENT",
    -104: "MKPP_ERROR_INVALID_STATE",
    -105: "MKPP_ERROR_CONVERGENCE",
    -106: "MKPP_ERROR_NOT_FOUND",
    -107: "MKPP_ERROR_DEVICE",
}
CELL_STATUS = {0: "SUCCESS", 1: "ERR_SINGULAR_MATRIX", 2: "ERR_NON_FINITE_STATE",
               3: "ERR_CONVERGENCE_FAILURE", 4: "ERR_NUMERICAL_FAILURE", 5: "ERR_CHECKPOINT_OVERFLOW"}
MODES = {"plain": 0, "persistent": 1}


class MkppError(RuntimeError):
    def __init__(self, code: int, message: str = ""):
        self.code = code
        super().__init__(f"{ERRORS.get(code, code)}: {message}" if message else ERRORS.get(code, str(code)))


_vp, _sz, _i, _d = C.c_void_p, C.c_size_t, C.c_int, C.c_double

# (name, restype, argtypes) of every symbol include/mkpp.h declares.
SIGNATURES = [
    ("mkpp_create_handle", _i, [_vp, _sz]),
    ("mkpp_destroy_handle", _i, [_vp]),
    ("mkpp_initialize", _i, [_vp]),
    ("mkpp_get_species_count", _i, [_vp, _vp]),
    ("mkpp_get_reaction_count", _i, [_vp, _vp]),
    ("mkpp_get_photolysis_count", _i, [_vp, _vp]),
    ("mkpp_get_species_index", _i, [_vp, C.c_char_p, _vp]),
    ("mkpp_get_photolysis_index", _i, [_vp, C.c_char_p, _vp]),
    ("mkpp_set_state_ptrs", _i, [_vp, _vp, _vp, _vp, _vp]),
    ("mkpp_set_rate_parameter_ptrs", _i, [_vp, _vp, _sz]),
    ("mkpp_set_photolysis_ptrs", _i, [_vp, _vp]),
    ("mkpp_set_cloud_water_ptr", _i, [_vp, _vp]),
    ("mkpp_set_aerosol_ptrs", _i, [_vp, _vp, _vp]),
    ("mkpp_integrate", _i, [_vp, _d]),
    ("mkpp_evaluate_rates", _i, [_vp, _vp]),
    ("mkpp_evaluate_jacobian", _i, [_vp, _vp]),
    ("mkpp_evaluate_jacobian_vector", _i, [_vp, _vp, _vp]),
    ("mkpp_evaluate_jacobian_transpose_vector", _i, [_vp, _vp, _vp]),
    ("mkpp_get_last_error", _i, [_vp, C.c_char_p, _sz]),
    ("mkpp_set_initial_step_seed", _i, [_vp, _d]),
    ("mkpp_set_max_attempts", _i, [_vp, _i]),
    ("mkpp_get_cell_stats", _i, [_vp, _vp, _vp, _vp]),
    ("mkpp_mechanism_name", _i, [_vp]),
    ("mkpp_mechanism_sizes", _i, [_vp, _vp, _vp, _vp, _vp]),
    ("mkpp_gpu_workspace_bytes", _sz, [_sz]),
    ("mkpp_set_launch_tuning", _i, [_i, _i, _i]),
    ("mkpp_gpu_rate_constants", _i, [_sz, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp, _vp, _vp]),
    ("mkpp_gpu_integrate_k", _i, [_sz, _vp, _vp, _sz, _i, _d, _d, _i, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    ("mkpp_gpu_integrate_logged", _i, [_sz, _vp, _vp, _i, _d, _d, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp, _sz,
                                       _vp]),
    ("mkpp_gpu_evaluate_rates", _i, [_sz, _vp, _vp, _vp, _vp]),
    ("mkpp_gpu_evaluate_jacobian", _i, [_sz, _vp, _vp, _vp, _vp]),
    ("mkpp_gpu_adjoint_workspace_bytes", _sz, [_sz]),
    ("mkpp_gpu_integrate_checkpoint", _i, [_sz, _vp, _vp, _d, _d, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz,
                                           _vp]),
    ("mkpp_gpu_integrate_replay", _i, [_sz, _vp, _vp, _i, _vp, _vp, _vp, _sz, _vp]),
    ("mkpp_gpu_adjoint", _i, [_sz, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    ("mkpp_set_cost_order", _i, [_vp, _i]),
    ("mkpp_set_split_launch", _i, [_i, _i]),
    ("mkpp_set_dt_carryover", _i, [_vp, _i]),
    ("mkpp_gpu_integrate_carry", _i, [_sz, _vp, _vp, _sz, _i, _d, _d, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _sz,
                                      _vp]),
    ("mkpp_mechanism_flags", _i, [_vp, _vp]),
    ("mkpp_mechanism_tolerances", _i, [_vp, _vp]),
    ("mkpp_set_tail_parking", _i, [_i]),
    ("mkpp_gpu_tangent_workspace_bytes", _sz, [_sz]),
    ("mkpp_gpu_tangent", _i, [_sz, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    ("mkpp_gpu_integrate_noalloc", _i, [_sz, _vp, _vp, _sz, _i, _d, _d, _i, _vp, _vp, _vp, _vp]),
]

_LIBS: dict[str, C.CDLL] = {}


def library_path(mechanism: str) -> Path:
    return LIB_DIR / f"libmkpp_{mechanism}.so"


def load_library(mechanism: str) -> C.CDLL:
    """Load libmkpp_<mechanism>.so, raising if it was not built."""
    if mechanism in _LIBS:
        return _LIBS[mechanism]
    path = library_path(mechanism)
    if not path.exists():
        raise RuntimeError(f"{path} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"`")
    lib = C.CDLL(str(path))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIBS[mechanism] = lib
    return lib


@dataclass(frozen=True)
class Sizes:
    species: int
    variable: int
    reactions: int
    rate_parameters: int
    lu_slots: int


def sizes(mechanism: str) -> Sizes:
    lib = load_library(mechanism)
    v = [C.c_int() for _ in range(5)]
    lib.mkpp_mechanism_sizes(*[C.byref(x) for x in v])
    return Sizes(*[x.value for x in v])


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch tensor


class MechanismContext:
    """Host-buffer handle, the C++ ``MechanismContext`` of the reference host API."""

    def __init__(self, mechanism: str, num_cells: int):
        self.mechanism = mechanism
        self.lib = load_library(mechanism)
        self.num_cells = int(num_cells)
        h = C.c_void_p()
        self._check(self.lib.mkpp_create_handle(C.byref(h), C.c_size_t(self.num_cells)), handle=False)
        self.handle = h
        self._check(self.lib.mkpp_initialize(self.handle))
        self._bound = []
        self.sizes = sizes(mechanism)

    def _check(self, rc: int, handle: bool = True):
        if rc != MKPP_SUCCESS:
            msg = self.last_error() if handle else ""
            raise MkppError(rc, msg)

    def last_error(self) -> str:
        buf = C.create_string_buffer(1024)
        self.lib.mkpp_get_last_error(self.handle, buf, C.c_size_t(len(buf)))
        return buf.value.decode()

    def close(self):
        if getattr(self, "handle", None):
            self.lib.mkpp_destroy_handle(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- metadata --------------------------------------------------------
    def species_index(self, name: str) -> int:
        idx = C.c_int()
        self._check(self.lib.mkpp_get_species_index(self.handle, name.encode(), C.byref(idx)))
        return idx.value

    def photolysis_index(self, name: str) -> int:
        idx = C.c_int()
        self._check(self.lib.mkpp_get_photolysis_index(self.handle, name.encode(), C.byref(idx)))
        return idx.value

    # --- binding (arrays must stay alive while bound) --------------------
    @staticmethod
    def _host(a, shape=None):
        if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
            raise TypeError("host arrays must be C-contiguous float64 numpy arrays")
        if shape is not None and a.shape != shape:
            raise ValueError(f"expected shape {shape}, got {a.shape}")
        return a

    def set_state(self, conc, temp, pressure, air_density):
        n = self.num_cells
        conc = self._host(conc, (self.sizes.species, n))
        arrs = [conc, self._host(temp, (n,)), self._host(pressure, (n,)), self._host(air_density, (n,))]
        self._bound += arrs
        self._check(self.lib.mkpp_set_state_ptrs(self.handle, *[_ptr(a) for a in arrs]))

    def set_rate_parameters(self, values):
        values = self._host(values)
        self._bound.append(values)
        count = values.shape[0] if values.ndim == 2 else 0
        self._check(self.lib.mkpp_set_rate_parameter_ptrs(self.handle, _ptr(values), C.c_size_t(count)))

    def set_photolysis(self, values):
        values = self._host(values)
        self._bound.append(values)
        self._check(self.lib.mkpp_set_photolysis_ptrs(self.handle, _ptr(values)))

    def set_cloud_water(self, values):
        values = self._host(values, (self.num_cells,))
        self._bound.append(values)
        self._check(self.lib.mkpp_set_cloud_water_ptr(self.handle, _ptr(values)))

    def set_aerosol(self, relative_humidity=None, surface_area=None):
        for a in (relative_humidity, surface_area):
            if a is not None:
                self._bound.append(self._host(a, (self.num_cells,)))
        self._check(self.lib.mkpp_set_aerosol_ptrs(self.handle, _ptr(relative_humidity), _ptr(surface_area)))

    def set_initial_step_seed(self, seed: float):
        self._check(self.lib.mkpp_set_initial_step_seed(self.handle, C.c_double(seed)))

    def set_max_attempts(self, n: int):
        self._check(self.lib.mkpp_set_max_attempts(self.handle, C.c_int(n)))

    def set_cost_order(self, enable: bool = True):
        """Hand out the previous call's most expensive cells first."""
        self._check(self.lib.mkpp_set_cost_order(self.handle, C.c_int(1 if enable else 0)))

    def set_dt_carryover(self, enable: bool = True):
        """Start each call at the step size the previous call ended with
        (changes results within the tolerances; off by default)."""
        self._check(self.lib.mkpp_set_dt_carryover(self.handle, C.c_int(1 if enable else 0)))

    # --- compute ---------------------------------------------------------
    def integrate(self, dt: float):
        self._check(self.lib.mkpp_integrate(self.handle, C.c_double(dt)))

    def evaluate_rates(self) -> np.ndarray:
        out = np.zeros((self.sizes.species, self.num_cells))
        self._check(self.lib.mkpp_evaluate_rates(self.handle, _ptr(out)))
        return out

    def evaluate_jacobian(self) -> np.ndarray:
        """Dense Jacobian as (N_col, N_row, cells): jac[col, row, cell] = dF_row/dC_col."""
        ns = self.sizes.species
        out = np.zeros((ns, ns, self.num_cells))
        self._check(self.lib.mkpp_evaluate_jacobian(self.handle, _ptr(out)))
        return out

    def evaluate_jacobian_vector(self, delta, transpose: bool = False) -> np.ndarray:
        """J delta (or J^T delta) per cell, (species, cells) arrays."""
        delta = self._host(delta, (self.sizes.species, self.num_cells))
        out = np.zeros((self.sizes.species, self.num_cells))
        fn = self.lib.mkpp_evaluate_jacobian_transpose_vector if transpose else self.lib.mkpp_evaluate_jacobian_vector
        self._check(fn(self.handle, _ptr(delta), _ptr(out)))
        return out

    def cell_stats(self):
        n = self.num_cells
        st, acc, rej = (np.zeros(n, np.int32) for _ in range(3))
        self._check(self.lib.mkpp_get_cell_stats(self.handle, _ptr(st), _ptr(acc), _ptr(rej)))
        return st, acc, rej


class DeviceSolver:
    """Device-pointer entry points on torch CUDA tensors (current stream)."""

    def __init__(self, mechanism: str):
        import torch

        self.torch = torch
        self.mechanism = mechanism
        self.lib = load_library(mechanism)
        self.sizes = sizes(mechanism)
        self._ws = None

    def _stream(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def _check(self, rc):
        if rc != MKPP_SUCCESS:
            raise MkppError(rc)

    def _dev(self, t, shape=None, dtype=None):
        torch = self.torch
        if t is None:
            return None
        if not (t.is_cuda and t.is_contiguous()):
            raise ValueError("device arrays must be contiguous CUDA tensors")
        if dtype is not None and t.dtype != dtype:
            raise TypeError(f"expected {dtype}, got {t.dtype}")
        if shape is not None and tuple(t.shape) != tuple(shape):
            raise ValueError(f"expected shape {tuple(shape)}, got {tuple(t.shape)}")
        return t

    def set_tuning(self, register_variant=0, blocks_per_sm=0, defer_after=-1):
        self._check(self.lib.mkpp_set_launch_tuning(C.c_int(register_variant), C.c_int(blocks_per_sm),
                                                    C.c_int(defer_after)))
        self._ws = None

    def set_split_launch(self, cells: int, sms: int):
        """The first `cells` entries of a launch's cell order go to whole
        warps on `sms` reserved SMs, in the persistent launch (0: off)."""
        self._check(self.lib.mkpp_set_split_launch(C.c_int(cells), C.c_int(sms)))
        self._ws = None

    def set_tail_parking(self, min_attempts: int):
        """Park the last cells on lanes after min_attempts attempts (0: off)."""
        self._check(self.lib.mkpp_set_tail_parking(C.c_int(min_attempts)))

    def workspace(self, n: int):
        torch = self.torch
        need = int(self.lib.mkpp_gpu_workspace_bytes(C.c_size_t(n)))
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.zeros(need + 256, dtype=torch.uint8, device="cuda")
        return self._ws

    def rate_constants(self, conc, temp=None, rho=None, rh=None, clw=None, param=None, ktab=None, status=None):
        torch = self.torch
        ns, n = conc.shape
        f64 = torch.float64
        self._dev(conc, (self.sizes.species, n), f64)
        for a in (temp, rho, rh, clw):
            self._dev(a, (n,), f64)
        if param is not None:
            self._dev(param, (self.sizes.rate_parameters, n), f64)
        if ktab is None:
            ktab = torch.empty((self.sizes.reactions, n), dtype=f64, device=conc.device)
        if status is None:
            status = torch.zeros(n, dtype=torch.int32, device=conc.device)
        rc = self.lib.mkpp_gpu_rate_constants(
            C.c_size_t(n), _ptr(conc), _ptr(temp), _ptr(rho), _ptr(rh), _ptr(clw), _ptr(param),
            C.c_size_t(self.sizes.rate_parameters if param is not None else 0), _ptr(ktab), _ptr(status),
            self._stream())
        self._check(rc)
        return ktab, status

    def integrate_k(self, conc, ktab, dt, steps=1, seed=None, max_attempts=20000, mode="persistent",
                    status=None, accepted=None, rejected=None, order=None, k_step_stride=0, dt_carry=None):
        """dt_carry: optional float64 [cells] device tensor, in/out, for
        step-size carry-over across calls (mkpp_gpu_integrate_carry)."""
        torch = self.torch
        ns, n = conc.shape
        if seed is None:
            seed = self.default_seed
        ws = self.workspace(n)
        common = (C.c_size_t(n), _ptr(conc), _ptr(ktab), C.c_size_t(k_step_stride), C.c_int(steps), C.c_double(dt),
                  C.c_double(seed), C.c_int(max_attempts), C.c_int(MODES[mode]), _ptr(order), _ptr(status),
                  _ptr(accepted), _ptr(rejected))
        if dt_carry is None:
            rc = self.lib.mkpp_gpu_integrate_k(*common, _ptr(ws), C.c_size_t(ws.numel()), self._stream())
        else:
            if dt_carry.dtype != torch.float64 or dt_carry.shape != (n,) or not dt_carry.is_contiguous():
                raise ValueError("dt_carry must be a contiguous float64 tensor of one value per cell")
            rc = self.lib.mkpp_gpu_integrate_carry(*common, _ptr(dt_carry), _ptr(ws), C.c_size_t(ws.numel()),
                                                  self._stream())
        self._check(rc)

    def integrate(self, conc, dt, steps=1, temp=None, rho=None, rh=None, clw=None, param=None, seed=None,
                  max_attempts=20000, mode="persistent"):
        """Integrate in place; returns (status, accepted, rejected) int32 tensors."""
        torch = self.torch
        n = conc.shape[1]
        ktab, status = self.rate_constants(conc, temp, rho, rh, clw, param)
        acc = torch.zeros(n, dtype=torch.int32, device=conc.device)
        rej = torch.zeros(n, dtype=torch.int32, device=conc.device)
        self.integrate_k(conc, ktab, dt, steps, seed, max_attempts, mode, status, acc, rej)
        return status, acc, rej

    def integrate_logged(self, conc, ktab, dt, steps=1, seed=None, max_attempts=20000, log_cap=4096):
        torch = self.torch
        n = conc.shape[1]
        if seed is None:
            seed = self.default_seed
        dev = conc.device
        status = torch.zeros(n, dtype=torch.int32, device=dev)
        acc = torch.zeros(n, dtype=torch.int32, device=dev)
        rej = torch.zeros(n, dtype=torch.int32, device=dev)
        lh = torch.zeros((log_cap, n), dtype=torch.float64, device=dev)
        la = torch.zeros((log_cap, n), dtype=torch.uint8, device=dev)
        ln = torch.zeros(n, dtype=torch.int32, device=dev)
        ws = self.workspace(n)
        rc = self.lib.mkpp_gpu_integrate_logged(
            C.c_size_t(n), _ptr(conc), _ptr(ktab), C.c_int(steps), C.c_double(dt), C.c_double(seed),
            C.c_int(max_attempts), _ptr(status), _ptr(acc), _ptr(rej), _ptr(lh), _ptr(la), _ptr(ln),
            C.c_int(log_cap), _ptr(ws), C.c_size_t(ws.numel()), self._stream())
        self._check(rc)
        return {"status": status, "accepted": acc, "rejected": rej, "log_h": lh, "log_acc": la, "log_n": ln}

    def evaluate_rates(self, conc, ktab):
        torch = self.torch
        n = conc.shape[1]
        out = torch.empty((self.sizes.species, n), dtype=torch.float64, device=conc.device)
        self._check(self.lib.mkpp_gpu_evaluate_rates(C.c_size_t(n), _ptr(conc), _ptr(ktab), _ptr(out),
                                                     self._stream()))
        return out

    def evaluate_jacobian(self, conc, ktab):
        torch = self.torch
        n = conc.shape[1]
        ns = self.sizes.species
        out = torch.empty((ns, ns, n), dtype=torch.float64, device=conc.device)
        self._check(self.lib.mkpp_gpu_evaluate_jacobian(C.c_size_t(n), _ptr(conc), _ptr(ktab), _ptr(out),
                                                        self._stream()))
        return out

    @property
    def default_seed(self) -> float:
        from .emitter.plan import load_raw

        return float(load_raw(self.mechanism)["initial_step_seed"])

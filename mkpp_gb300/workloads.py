"""Seeded synthetic cell populations for the benchmark and parity workloads.

The reference publishes no dataset for this path; these draws stand in for
its scenarios with the shapes, sizes and value ranges of the workloads the
solver is measured on.  Every array is float64, species-major with the cell
index innermost (LayoutLeft).  All draws come from ``numpy.random.Generator``
seeded with 2718.

Workloads (cells, host steps x dt):

* ``chapman``       4096 cells, 1 x 3600 s.  O and O3 log-uniform in
  [1e2, 1e13] molec/cm3, T ~ U[190, 310] K, p ~ U[1e3, 1e5] Pa,
  M = p / (k_B T) * 1e-6, O2 = 0.21 M, J1, J3 ~ U[0, 1e-2] 1/s.
* ``small_strato``  65536 cells, 12 x 300 s.  Species log-uniform in [1, 1e12],
  O2 = 0.21 M, half the cells night (all J = 0), half day (J log-uniform in
  [1e-8, 1e-2]).
* ``saprc99``       262144 cells, 24 x 600 s.  Species log-uniform in
  [1e-2, 1e12]; NO, NO2 and the VOC classes scaled by a per-cell factor
  log-uniform in [0.01, 100]; AIR = M = p / (k_B T) * 1e-6, O2 = 0.21 M,
  N2 = 0.78 M, H2O from RH ~ U[0.1, 0.9]; T ~ U[250, 315] K.  Photolysis
  J_r(t) = Jmax_r * max(cos(2 pi t / 86400 + phi_c), 0) with a per-cell phase
  phi_c ~ U[0, 2 pi) (diurnal cosine of the solar zenith angle) and per-slot
  maxima Jmax_r log-uniform in [1e-6, 1e-2] 1/s (NO2 -> 8e-3 1/s).
* ``ts1``           1048576 cells, 6 x 600 s, mol/m3 units (molec/cm3 / 6.02214076e17),
  40 % night, 30 % clean (NOx x 0.01), 30 % polluted (NOx x 100).  Species
  log-uniform in [1e-2, 1e12] molec/cm3, photolysis as ``saprc99``, the user
  and heterogeneous rate slots from the reference's TS1 benchmark inputs.
  Its plan's atol is 1 molec/cm3 expressed in mol/m3 (1.66e-18), rtol 1e-3:
  the tolerances of the other workloads in TS1's units.

Further mechanisms the reference ships (no benchmark configuration; parity
cases only):

* ``saprc99_mini``, ``saprcnov``  65536 cells, 24 x 600 s, drawn as
  ``saprc99`` (background species AIR, M, O2, N2, H2O, CH4, H2, CO2 set from
  p, T and RH where the mechanism has them; saprcnov's fixed RO2 log-uniform
  in [1e6, 1e9]); the NO2 photolysis slot at 8e-3 1/s.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .emitter.plan import load_raw

SEED = 2718
K_B = 1.380649e-23          # J/K
AVOGADRO = 6.02214076e23
R_GAS = 8.314462618         # J/(mol K)

VOC_SAPRC99 = ("HCHO", "CCHO", "RCHO", "ACET", "MEK", "ETHENE", "ISOPRENE", "ALK1", "ALK2", "ALK3",
               "ALK4", "ALK5", "ARO1", "ARO2", "OLE1", "OLE2", "TERP", "MEOH", "CO")


@dataclass
class Workload:
    name: str
    mechanism: str
    conc: np.ndarray          # (NS, n)
    temp: np.ndarray          # (n,)
    pressure: np.ndarray      # (n,)
    rho: np.ndarray           # (n,)
    rh: np.ndarray            # (n,)
    param: np.ndarray         # (NP, n)
    dt: float
    host_steps: int
    phase: np.ndarray | None = None      # diurnal phase per cell (saprc99, ts1)
    jmax: np.ndarray | None = None       # (NP,) photolysis maxima
    extra: dict = field(default_factory=dict)

    @property
    def ncells(self) -> int:
        return self.conc.shape[1]

    def param_at(self, host_step: int) -> np.ndarray:
        """Runtime parameters during host step `host_step` (diurnal forcing)."""
        if self.phase is None:
            return self.param
        t = host_step * self.dt
        sun = np.maximum(np.cos(2.0 * np.pi * t / 86400.0 + self.phase), 0.0)
        out = self.param.copy()
        nph = len(self.jmax)
        out[:nph] = self.jmax[:, None] * sun[None, :]
        return out

    def subset(self, n: int) -> "Workload":
        sl = slice(0, n)
        return Workload(self.name, self.mechanism, np.ascontiguousarray(self.conc[:, sl]), self.temp[sl].copy(),
                        self.pressure[sl].copy(), self.rho[sl].copy(), self.rh[sl].copy(),
                        np.ascontiguousarray(self.param[:, sl]), self.dt, self.host_steps,
                        None if self.phase is None else self.phase[sl].copy(), self.jmax, dict(self.extra))


def _loguniform(rng, lo, hi, size):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size))


def _species_index(raw):
    return {s: i for i, s in enumerate(raw["species"])}


def chapman(ncells: int = 4096, seed: int = SEED) -> Workload:
    raw = load_raw("chapman")
    rng = np.random.default_rng(seed)
    ix = _species_index(raw)
    T = rng.uniform(190.0, 310.0, ncells)
    p = rng.uniform(1e3, 1e5, ncells)
    M = p / (K_B * T) * 1e-6
    conc = np.zeros((len(raw["species"]), ncells))
    conc[ix["O"]] = _loguniform(rng, 1e2, 1e13, ncells)
    conc[ix["O3"]] = _loguniform(rng, 1e2, 1e13, ncells)
    conc[ix["M"]] = M
    conc[ix["O2"]] = 0.21 * M
    param = rng.uniform(0.0, 1e-2, (raw["num_rate_parameters"], ncells))
    return Workload("chapman", "chapman", conc, T, p, M.copy(), np.full(ncells, 0.5), param, 3600.0, 1)


def small_strato(ncells: int = 65536, seed: int = SEED) -> Workload:
    raw = load_raw("small_strato")
    rng = np.random.default_rng(seed)
    ix = _species_index(raw)
    T = rng.uniform(190.0, 310.0, ncells)
    p = rng.uniform(1e3, 1e5, ncells)
    M = p / (K_B * T) * 1e-6
    conc = _loguniform(rng, 1.0, 1e12, (len(raw["species"]), ncells))
    conc[ix["M"]] = M
    conc[ix["O2"]] = 0.21 * M
    npar = raw["num_rate_parameters"]
    param = _loguniform(rng, 1e-8, 1e-2, (npar, ncells))
    night = np.zeros(ncells, bool)
    night[: ncells // 2] = True
    rng.shuffle(night)
    param[:, night] = 0.0
    return Workload("small_strato", "small_strato", conc, T, p, M.copy(), np.full(ncells, 0.5), param, 300.0, 12,
                    extra={"night": night})


def _jmax(raw, rng, no2_slot=None):
    nph = raw["num_photolysis"]
    jmax = _loguniform(rng, 1e-6, 1e-2, nph)
    if no2_slot is not None:
        jmax[no2_slot] = 8e-3
    return jmax


def saprc99(ncells: int = 262144, seed: int = SEED) -> Workload:
    raw = load_raw("saprc99")
    rng = np.random.default_rng(seed)
    ix = _species_index(raw)
    ns = len(raw["species"])
    T = rng.uniform(250.0, 315.0, ncells)
    p = rng.uniform(5e4, 1.05e5, ncells)
    M = p / (K_B * T) * 1e-6
    rh = rng.uniform(0.1, 0.9, ncells)
    conc = _loguniform(rng, 1e-2, 1e12, (ns, ncells))
    factor = _loguniform(rng, 0.01, 100.0, ncells)
    for s in ("NO", "NO2", *VOC_SAPRC99):
        conc[ix[s]] *= factor
    conc[ix["AIR"]] = M
    conc[ix["M"]] = M
    conc[ix["O2"]] = 0.21 * M
    conc[ix["N2"]] = 0.78 * M
    # Water vapour from relative humidity (Magnus saturation pressure).
    es = 610.94 * np.exp(17.625 * (T - 273.15) / (T - 30.11))
    conc[ix["H2O"]] = rh * es / (K_B * T) * 1e-6
    conc[ix["CH4"]] = 1.8e-6 * M
    conc[ix["H2"]] = 5.5e-7 * M
    phase = rng.uniform(0.0, 2.0 * np.pi, ncells)
    # Slot 0 is NO2 + hv -> NO + O3P in this mechanism's photolysis order.
    jmax = _jmax(raw, rng, no2_slot=0)
    param = np.zeros((raw["num_rate_parameters"], ncells))
    w = Workload("saprc99", "saprc99", conc, T, p, M.copy(), rh, param, 600.0, 24, phase=phase, jmax=jmax)
    w.param = w.param_at(0)
    return w


def ts1(ncells: int = 1048576, seed: int = SEED) -> Workload:
    raw = load_raw("ts1")
    rng = np.random.default_rng(seed)
    ix = _species_index(raw)
    ns = len(raw["species"])
    T = rng.uniform(250.0, 315.0, ncells)
    p = rng.uniform(5e4, 1.05e5, ncells)
    to_mol_m3 = 1.0 / 6.02214076e17           # molec/cm3 -> mol/m3
    M = p / (K_B * T) * 1e-6
    conc = _loguniform(rng, 1e-2, 1e12, (ns, ncells)) * to_mol_m3
    kind = rng.choice(3, size=ncells, p=[0.4, 0.3, 0.3])   # 0 night, 1 clean, 2 polluted
    nox = np.where(kind == 1, 0.01, np.where(kind == 2, 100.0, 1.0))
    for s in ("NO", "NO2"):
        conc[ix[s]] *= nox
    conc[ix["M"]] = M * to_mol_m3
    conc[ix["O2"]] = 0.21 * M * to_mol_m3
    conc[ix["N2"]] = 0.78 * M * to_mol_m3
    phase = rng.uniform(0.0, 2.0 * np.pi, ncells)
    phase[kind == 0] = np.pi                     # night cells: sun below horizon all run
    jmax = _jmax(raw, rng)
    param = np.zeros((raw["num_rate_parameters"], ncells))
    # The slots after the photolysis rates are user and heterogeneous rate
    # constants addressed by reaction index; every cell takes the values of
    # the reference's TS1 benchmark inputs.
    nph = raw["num_photolysis"]
    param[nph:] = ts1_user_rates(raw)[nph:, None]
    w = Workload("ts1", "ts1", conc, T, p, (M * to_mol_m3), np.full(ncells, 0.5), param, 600.0, 6,
                 phase=phase, jmax=jmax, extra={"kind": kind})
    w.param = w.param_at(0)
    return w


def ts1_user_rates(raw=None) -> np.ndarray:
    """TS1's runtime parameter row of the reference's native benchmark run
    (``benchmarks/solver_comparison/runners/mkpp/ts1_binding_data.hpp:246``,
    kept as the ``parameters`` of ``tests/golden/ts1_kokkos_2x300.json``).
    Slots 361-373, 499 and 529-546 are nonzero there: uptake on aerosol and
    heterogeneous halogen reactions, in 1/s or m3/(mol s)."""
    import json
    from pathlib import Path

    raw = raw or load_raw("ts1")
    path = Path(__file__).resolve().parent.parent / "tests" / "golden" / "ts1_kokkos_2x300.json"
    row = np.asarray(json.loads(path.read_text())["parameters"], dtype=np.float64)
    assert row.shape == (raw["num_rate_parameters"],)
    return row


def _photolysis_slot(raw, species):
    """Runtime parameter slot of the photolysis whose only reactant is `species`."""
    ix = _species_index(raw)[species]
    for ph in raw["photolysis_reactions"]:
        r = raw["reactions"][ph["reaction_idx"]]
        if [s for s, _ in r["reactants"]] == [ix]:
            return ph["photo_idx"]
    return None


def _background(raw, conc, M, T, rh):
    """Air, its major components and the long-lived background species."""
    ix = _species_index(raw)
    es = 610.94 * np.exp(17.625 * (T - 273.15) / (T - 30.11))     # Magnus, Pa
    fixed = {"AIR": M, "M": M, "O2": 0.21 * M, "N2": 0.78 * M, "H2O": rh * es / (K_B * T) * 1e-6,
             "CH4": 1.8e-6 * M, "H2": 5.5e-7 * M, "CO2": 4.2e-4 * M}
    for name, v in fixed.items():
        if name in ix:
            conc[ix[name]] = v


def _saprc_family(name: str, ncells: int, seed: int) -> Workload:
    raw = load_raw(name)
    rng = np.random.default_rng(seed)
    ix = _species_index(raw)
    T = rng.uniform(250.0, 315.0, ncells)
    p = rng.uniform(5e4, 1.05e5, ncells)
    M = p / (K_B * T) * 1e-6
    rh = rng.uniform(0.1, 0.9, ncells)
    conc = _loguniform(rng, 1e-2, 1e12, (len(raw["species"]), ncells))
    factor = _loguniform(rng, 0.01, 100.0, ncells)
    for s in ("NO", "NO2", *VOC_SAPRC99):
        if s in ix:
            conc[ix[s]] *= factor
    _background(raw, conc, M, T, rh)
    if "RO2" in ix and raw["fixed"][ix["RO2"]]:
        conc[ix["RO2"]] = _loguniform(rng, 1e6, 1e9, ncells)
    phase = rng.uniform(0.0, 2.0 * np.pi, ncells)
    jmax = _jmax(raw, rng, no2_slot=_photolysis_slot(raw, "NO2"))
    param = np.zeros((raw["num_rate_parameters"], ncells))
    w = Workload(name, name, conc, T, p, M.copy(), rh, param, 600.0, 24, phase=phase, jmax=jmax)
    w.param = w.param_at(0)
    return w


def saprc99_mini(ncells: int = 65536, seed: int = SEED) -> Workload:
    return _saprc_family("saprc99_mini", ncells, seed)


def saprcnov(ncells: int = 65536, seed: int = SEED) -> Workload:
    return _saprc_family("saprcnov", ncells, seed)


BUILDERS = {"chapman": chapman, "small_strato": small_strato, "saprc99": saprc99, "ts1": ts1,
            "saprc99_mini": saprc99_mini, "saprcnov": saprcnov}


# Libraries of a mechanism built with another tableau or other tolerances
# draw that mechanism's workload.
ALIASES = {"chapman_rodas3": "chapman", "small_strato_rodas3": "small_strato", "chapman_shipped": "chapman"}


def make(name: str, ncells: int | None = None, seed: int = SEED) -> Workload:
    base = ALIASES.get(name, name)
    fn = BUILDERS[base]
    w = fn(seed=seed) if ncells is None else fn(ncells, seed=seed)
    if base != name:
        w.name = w.mechanism = name
    return w

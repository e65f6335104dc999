"""Python face of the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` use this
module, and only as the checker / the timed CPU restatement; the product never imports it.

``liboracle.so`` (wbc_oracle.cpp) restates each reference kernel; this module binds it with
ctypes and adds ``OracleSim``, a numpy mirror of a whole coupled cell step in the reference's
operator-splitting order (simulation/simulator.py:58-81): field update (deposit -> combine ->
SOR to tolerance with the reference's check cadence, fields/diffusion.py:79-123 -> sample),
network step, lifecycle decide + inclusive scan + capacity check + placement
(cells/lifecycle.py:96-179), network inheritance, mechanics substeps
(cells/mechanics.py:112-122). Scalar parameters are rounded to float32 from the same double
expressions the reference passes to its kernels.
"""

from __future__ import annotations

import ctypes
import time
from ctypes import c_double, c_float, c_int32, c_int64, c_void_p
from dataclasses import dataclass, field

import numpy as np

from oracle.build import build as _build

_lib = None


class SorParams(ctypes.Structure):
    _fields_ = [("nx", c_int32), ("ny", c_int32), ("nz", c_int32), ("bc_x", c_int32), ("bc_y", c_int32),
                ("bc_z", c_int32), ("omega", c_float), ("dx2_over_D", c_float), ("uptake_max", c_float),
                ("michaelis_k", c_float), ("reference", c_float), ("has_source", c_int32), ("source_k", c_float)]


class LifecycleParamsC(ctypes.Structure):
    _fields_ = [("dt", c_float), ("death_rate", c_float), ("anoxic_death_rate", c_float), ("division_rate", c_float),
                ("inhibition_threshold", c_int32), ("hypoxia_threshold", c_float), ("death_threshold", c_float),
                ("glucose_threshold", c_float), ("glucose_death_threshold", c_float),
                ("necrosis_requires_glucose", c_int32), ("phenotype_model", c_int32), ("apoptosis_rate", c_float),
                ("necrosis_rate", c_float)]


class ProgramC(ctypes.Structure):
    _fields_ = [("n_nodes", c_int32), ("n_words", c_int32), ("n_ops", c_int32), ("n_updatable", c_int32),
                ("ops", c_void_p), ("args", c_void_p), ("start", c_void_p), ("length", c_void_p),
                ("updatable", c_void_p)]


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(_build()))
        _lib.orc_num_threads.restype = c_int32
        _lib.orc_division_scan.restype = c_int32
    return _lib


def P(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return a.ctypes.data_as(c_void_p)


def f32(x) -> c_float:
    return c_float(float(np.float32(x)))


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())


# ---- per-kernel wrappers ------------------------------------------------------------------------------
def rng_init(seed: int, capacity: int) -> np.ndarray:
    out = np.zeros(capacity, dtype=np.uint32)
    lib().orc_rng_init(c_int32(seed), P(out), c_int64(capacity))
    return out


def rng_uniform(state: np.ndarray, draws: int) -> np.ndarray:
    out = np.zeros((state.size, draws), dtype=np.float32)
    lib().orc_rng_uniform(c_int32(state.size), c_int32(draws), P(state), P(out))
    return out


def rng_sphere(state: np.ndarray) -> np.ndarray:
    out = np.zeros((state.size, 3), dtype=np.float32)
    lib().orc_rng_sphere(c_int32(state.size), P(state), P(out))
    return out


def expf(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    lib().orc_expf(c_int32(x.size), P(x), P(out))
    return out


def logf(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty_like(x)
    lib().orc_logf(c_int32(x.size), P(x), P(out))
    return out


def contact_substep(pos: np.ndarray, radius: np.ndarray, cell_size: float, dim: int, query_radius: float, rate: float,
                    dt: float, fp64: bool = False):
    """One contact substep in place on ``pos`` (n, 3); returns (velocity, neighbor_count)."""
    n = pos.shape[0]
    nc = np.zeros(n, dtype=np.int32)
    if fp64:
        assert pos.dtype == np.float64
        vel = np.zeros((n, 3), dtype=np.float64)
        r = np.ascontiguousarray(radius, dtype=np.float64)
        lib().orc_contact_substep_f64(c_int32(n), P(pos), P(r), f32(cell_size), c_int32(dim), c_double(query_radius),
                                      c_double(rate), c_double(dt), P(vel), P(nc))
    else:
        assert pos.dtype == np.float32
        vel = np.zeros((n, 3), dtype=np.float32)
        r = np.ascontiguousarray(radius, dtype=np.float32)
        lib().orc_contact_substep_f32(c_int32(n), P(pos), P(r), f32(cell_size), c_int32(dim), f32(query_radius),
                                      f32(rate), f32(dt), P(vel), P(nc))
    return vel, nc


@dataclass(frozen=True)
class Geometry:
    origin: tuple
    dx: float
    shape: tuple

    @property
    def nodes(self) -> int:
        return int(np.prod(self.shape))


def deposit(geom: Geometry, pos: np.ndarray, state: np.ndarray, acc: np.ndarray | None = None) -> np.ndarray:
    """int64 accumulator (4, nx, ny, nz) of trilinear fixed-point weights (added to ``acc``)."""
    nx, ny, nz = geom.shape
    if acc is None:
        acc = np.zeros((4, nx, ny, nz), dtype=np.int64)
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    state = np.ascontiguousarray(state, dtype=np.int32)
    o = geom.origin
    lib().orc_deposit(c_int32(nx), c_int32(ny), c_int32(nz), f32(o[0]), f32(o[1]), f32(o[2]), f32(1.0 / geom.dx),
                      c_int32(pos.shape[0]), P(pos), P(state), P(acc))
    return acc


def density_convert(geom: Geometry, acc: np.ndarray, weights=None):
    dens = np.zeros((4,) + tuple(geom.shape), dtype=np.float32)
    comb = None
    w = None
    if weights is not None:
        w = np.ascontiguousarray(weights, dtype=np.float32)
        comb = np.zeros(tuple(geom.shape), dtype=np.float32)
    lib().orc_density_convert(c_int64(geom.nodes), P(acc), f32(1.0 / geom.dx**3), P(dens), P(w), P(comb))
    return dens, comb


def combine(density: np.ndarray, weights) -> np.ndarray:
    w = [np.float32(x) for x in weights]
    return ((w[0] * density[0] + w[1] * density[1]) + w[2] * density[2]) + w[3] * density[3]


def sample(geom: Geometry, field_values: np.ndarray, pos: np.ndarray, fp64: bool = False) -> np.ndarray:
    nx, ny, nz = geom.shape
    o = geom.origin
    n = pos.shape[0]
    if fp64:
        f = np.ascontiguousarray(field_values, dtype=np.float64)
        p = np.ascontiguousarray(pos, dtype=np.float64)
        out = np.zeros(n, dtype=np.float64)
        lib().orc_sample_f64(c_int32(nx), c_int32(ny), c_int32(nz), c_double(o[0]), c_double(o[1]), c_double(o[2]),
                             c_double(1.0 / geom.dx), P(f), c_int32(n), P(p), P(out))
    else:
        f = np.ascontiguousarray(field_values, dtype=np.float32)
        p = np.ascontiguousarray(pos, dtype=np.float32)
        out = np.zeros(n, dtype=np.float32)
        lib().orc_sample_f32(c_int32(nx), c_int32(ny), c_int32(nz), f32(o[0]), f32(o[1]), f32(o[2]),
                             f32(1.0 / geom.dx), P(f), c_int32(n), P(p), P(out))
    return out


def sor_params(geom: Geometry, boundary, boundary_value: float, diffusion: float, uptake_max: float,
               michaelis_k: float, omega: float, has_source: int = 0, source_k: float = 1.0) -> SorParams:
    nx, ny, nz = geom.shape
    reference = boundary_value if boundary_value > 0.0 else 1.0
    return SorParams(nx=nx, ny=ny, nz=nz, bc_x=int(boundary[0]), bc_y=int(boundary[1]), bc_z=int(boundary[2]),
                     omega=omega, dx2_over_D=geom.dx**2 / diffusion, uptake_max=uptake_max, michaelis_k=michaelis_k,
                     reference=reference, has_source=has_source, source_k=source_k)


def sor_sweeps(params: SorParams, sweeps: int, fixed: np.ndarray, density: np.ndarray, values: np.ndarray,
               production: np.ndarray | None = None, source: np.ndarray | None = None, residual: bool = True,
               fp64: bool = False) -> float | None:
    """``sweeps`` red-black sweeps in place on ``values``; returns the residual when asked."""
    fixed = np.ascontiguousarray(fixed, dtype=np.int32)
    if fp64:
        res = np.zeros(1, dtype=np.float64)
        lib().orc_sor_sweeps_f64(ctypes.byref(params), c_int32(sweeps), P(fixed), P(density), P(production),
                                 P(source), P(values), P(res) if residual else None)
    else:
        res = np.zeros(1, dtype=np.float32)
        lib().orc_sor_sweeps_f32(ctypes.byref(params), c_int32(sweeps), P(fixed), P(density), P(production),
                                 P(source), P(values), P(res) if residual else None)
    return float(res[0]) if residual else None


def ftcs_step(params: SorParams, dt: float, fixed: np.ndarray, density: np.ndarray, values: np.ndarray,
              production=None, source=None) -> np.ndarray:
    out = np.empty_like(values)
    lib().orc_ftcs_step_f32(ctypes.byref(params), f32(dt), P(np.ascontiguousarray(fixed, dtype=np.int32)),
                            P(density), P(production), P(source), P(values), P(out))
    return out


def solve_steady_state(params: SorParams, settings, fixed, density, values, production=None, source=None,
                       fp64: bool = False):
    """Reference stopping rule: chunks of ``check_every`` sweeps, residual after each chunk."""
    sweeps = 0
    residual = float("inf")
    while sweeps < settings.max_sweeps:
        chunk = min(settings.check_every, settings.max_sweeps - sweeps)
        residual = sor_sweeps(params, chunk, fixed, density, values, production, source, True, fp64)
        sweeps += chunk
        if residual < settings.tolerance:
            return sweeps, residual, True
    return sweeps, residual, False


def lifecycle_params(params, dt: float) -> LifecycleParamsC:
    return LifecycleParamsC(dt=dt, death_rate=params.death_rate, anoxic_death_rate=params.anoxic_death_rate,
                            division_rate=params.division_rate,
                            inhibition_threshold=min(int(params.inhibition_threshold), 2**31 - 1),
                            hypoxia_threshold=params.hypoxia_threshold, death_threshold=params.death_threshold,
                            glucose_threshold=params.glucose_threshold,
                            glucose_death_threshold=params.glucose_death_threshold,
                            necrosis_requires_glucose=1 if params.necrosis_requires_glucose else 0,
                            phenotype_model=1 if params.phenotype_model == "network" else 0,
                            apoptosis_rate=params.apoptosis_rate, necrosis_rate=params.necrosis_rate)


def program(arrays: dict, n_nodes: int) -> tuple[ProgramC, list]:
    keep = [np.ascontiguousarray(arrays[k], dtype=np.int32) for k in ("ops", "args", "start", "length", "updatable")]
    p = ProgramC(n_nodes=n_nodes, n_words=(n_nodes + 63) // 64, n_ops=keep[0].size, n_updatable=keep[4].size,
                 ops=P(keep[0]), args=P(keep[1]), start=P(keep[2]), length=P(keep[3]), updatable=P(keep[4]))
    return p, keep


# ---- whole-step mirror --------------------------------------------------------------------------------
@dataclass
class OracleSim:
    """numpy mirror of a population (capacity-sized arrays) plus its optional fields and network."""

    capacity: int
    count: int
    seed: int
    position: np.ndarray
    radius: np.ndarray
    cell_state: np.ndarray
    cell_type: np.ndarray
    age: np.ndarray
    oxygen_local: np.ndarray
    glucose_local: np.ndarray
    rng_state: np.ndarray
    velocity: np.ndarray
    neighbor_count: np.ndarray
    divide_flag: np.ndarray
    division_offset: np.ndarray
    fate_flags: np.ndarray
    extra_local: dict = field(default_factory=dict)

    @classmethod
    def from_numpy(cls, positions, radii, capacity=None, seed=0, states=None) -> OracleSim:
        positions = np.asarray(positions, dtype=np.float32)
        n = positions.shape[0]
        cap = n if capacity is None else int(capacity)

        def padded(v, dtype, fill=0):
            buf = np.full((cap,) + np.shape(v)[1:], fill, dtype=dtype)
            buf[:n] = v
            return buf

        if states is None:
            states = np.zeros(n, dtype=np.int32)
        return cls(capacity=cap, count=n, seed=int(seed), position=padded(positions, np.float32),
                   radius=padded(np.asarray(radii, np.float32), np.float32),
                   cell_state=padded(np.asarray(states, np.int32), np.int32, 3),
                   cell_type=np.zeros(cap, np.int32), age=np.zeros(cap, np.float32),
                   oxygen_local=np.zeros(cap, np.float32), glucose_local=np.zeros(cap, np.float32),
                   rng_state=rng_init(seed, cap), velocity=np.zeros((cap, 3), np.float32),
                   neighbor_count=np.zeros(cap, np.int32), divide_flag=np.zeros(cap, np.int32),
                   division_offset=np.zeros(cap, np.int32), fate_flags=np.zeros(cap, np.int32))

    def local_field(self, name: str) -> np.ndarray:
        if name == "oxygen":
            return self.oxygen_local
        if name == "glucose":
            return self.glucose_local
        if name not in self.extra_local:
            self.extra_local[name] = np.zeros(self.capacity, np.float32)
        return self.extra_local[name]

    # mechanics (cells/mechanics.py:75-122)
    def contact_substep(self, cell_size: float, dim: int, query_radius: float, rate: float, dt: float) -> None:
        n = self.count
        if n == 0:
            return
        pos = np.ascontiguousarray(self.position[:n])
        vel, nc = contact_substep(pos, self.radius[:n], cell_size, dim, query_radius, rate, dt)
        self.position[:n] = pos
        self.velocity[:n] = vel
        self.neighbor_count[:n] = nc

    # lifecycle (cells/lifecycle.py:96-179)
    def decide_lifecycle(self, params, dt: float) -> None:
        n = self.count
        if n == 0:
            return
        lib().orc_lifecycle_decide(ctypes.byref(lifecycle_params(params, dt)), c_int32(n), P(self.cell_state),
                                   P(self.age), P(self.neighbor_count), P(self.oxygen_local), P(self.glucose_local),
                                   P(self.fate_flags), P(self.rng_state), P(self.divide_flag))

    def commit_divisions(self, params) -> int:
        n = self.count
        if n == 0:
            return 0
        total = int(lib().orc_division_scan(c_int32(n), P(self.divide_flag), P(self.division_offset)))
        if total == 0:
            return 0
        if n + total > self.capacity:
            raise OverflowError("capacity exceeded")
        lib().orc_place_daughters(c_int32(n), f32(params.placement_factor), P(self.divide_flag),
                                  P(self.division_offset), P(self.position), P(self.radius), P(self.cell_state),
                                  P(self.cell_type), P(self.age), P(self.oxygen_local), P(self.glucose_local),
                                  P(self.rng_state), P(self.velocity), P(self.neighbor_count), P(self.fate_flags))
        self.count = n + total
        return total


@dataclass
class OracleSpecies:
    """Mirror of one SpeciesField (fields/species.py:95-195) on an OracleSim."""

    geom: Geometry
    boundary: tuple
    boundary_value: float
    diffusion: float
    uptake_max: tuple
    michaelis_k: float
    settings: object
    production: tuple = (0.0, 0.0, 0.0, 0.0)
    name: str = "oxygen"
    values: np.ndarray = None
    fixed: np.ndarray = None

    def __post_init__(self):
        shape = tuple(self.geom.shape)
        self.values = np.full(shape, np.float32(self.boundary_value), dtype=np.float32)
        if self.fixed is None:
            self.fixed = np.zeros(shape, dtype=np.int32)
        self.density = np.zeros(shape, np.float32)
        self.prod = np.zeros(shape, np.float32)

    @property
    def uptake_scale(self) -> float:
        return max(self.uptake_max) if max(self.uptake_max) > 0.0 else 0.0

    @property
    def uptake_weights(self):
        s = self.uptake_scale
        return tuple(u / s if s > 0.0 else 0.0 for u in self.uptake_max)

    @property
    def produces(self) -> bool:
        return max(self.production) > 0.0

    def combine(self, densities: np.ndarray) -> None:
        self.density = combine(densities, self.uptake_weights)
        if self.produces:
            self.prod = combine(densities, self.production)

    def solve(self, source=None, source_k: float = 1.0):
        p = sor_params(self.geom, self.boundary, self.boundary_value, self.diffusion, self.uptake_scale,
                       self.michaelis_k, self.settings.omega, 1 if source is not None else 0, source_k)
        return solve_steady_state(p, self.settings, self.fixed, self.density, self.values,
                                  self.prod if self.produces else None, source)

    def sample_into(self, sim: OracleSim, out: np.ndarray) -> None:
        n = sim.count
        out[:n] = sample(self.geom, self.values, sim.position[:n])


def cell_step(sim: OracleSim, lifecycle, contact, dt_cells: float, dt_mechanics: float, species: OracleSpecies | None = None,
              dim: int = 128):
    """Mirror of simulation/simulator.py:58-81 (no network) on an OracleSim; returns
    (daughters, (sweeps, residual, converged) or None). ``contact`` needs ``query_radius`` and
    ``rate`` (a ContactParams)."""
    report = None
    if species is not None:
        n = sim.count
        acc = deposit(species.geom, sim.position[:n], sim.cell_state[:n])
        dens, _ = density_convert(species.geom, acc)
        species.combine(dens)
        report = species.solve()
        species.sample_into(sim, sim.oxygen_local)
    sim.decide_lifecycle(lifecycle, dt_cells)
    daughters = sim.commit_divisions(lifecycle)
    substeps = max(1, int(round(dt_cells / dt_mechanics)))
    for _ in range(substeps):
        sim.contact_substep(contact.query_radius, dim, contact.query_radius, contact.rate, dt_mechanics)
    return daughters, report


@dataclass
class OracleNetwork:
    """Mirror of a NetworkRuntime (network/runtime.py:89-228): program arrays, clamps, words."""

    arrays: dict  # the programs() arrays (ops, args, start, length, updatable, rates, p_on)
    n_nodes: int
    capacity: int
    update: str = "synchronous"
    updates_per_step: int = 1
    time_units_per_h: float = 10.0
    max_events: int = 20000
    clamps: tuple = ()  # (node index, source code 0-4, threshold, above)
    fate_nodes: tuple = (-1, -1, -1, -1)
    extra_names: tuple = ()

    def __post_init__(self):
        self.n_words = (self.n_nodes + 63) // 64
        self.words = np.zeros((self.capacity, self.n_words), dtype=np.uint64)
        self.prog, self._keep = program(self.arrays, self.n_nodes)
        c = self.clamps or ((0, 4, 0.0, 1),)
        self.c_node = np.array([x[0] for x in c], np.int32)
        self.c_source = np.array([x[1] for x in c], np.int32)
        self.c_thr = np.array([x[2] for x in c], np.float32)
        self.c_above = np.array([x[3] for x in c], np.int32)
        self.p_on = np.ascontiguousarray(self.arrays["p_on"], dtype=np.float32)
        self.rates = {k: np.ascontiguousarray(self.arrays[k], dtype=np.float32)
                      for k in ("rate_up_true", "rate_up_false", "rate_down_true", "rate_down_false")}

    def initialize(self, sim: OracleSim) -> None:
        lib().orc_network_initialize(ctypes.byref(self.prog), c_int32(sim.count), P(self.p_on), P(sim.rng_state),
                                     P(self.words))
        self.read_fates(sim)

    def read_fates(self, sim: OracleSim) -> None:
        lib().orc_network_read_fates(c_int32(sim.count), c_int32(self.n_words), *[c_int32(x) for x in self.fate_nodes],
                                     P(self.words), P(sim.fate_flags))

    def step(self, sim: OracleSim, dt_h: float) -> None:
        n = sim.count
        if len(self.clamps):
            extra = [sim.local_field(x) for x in self.extra_names[:2]]
            ea = extra[0] if len(extra) > 0 else sim.oxygen_local
            eb = extra[1] if len(extra) > 1 else sim.oxygen_local
            lib().orc_network_clamp_inputs(c_int32(n), c_int32(self.n_words), c_int32(len(self.clamps)),
                                           P(self.c_node), P(self.c_source), P(self.c_thr), P(self.c_above),
                                           P(sim.oxygen_local), P(sim.glucose_local), P(ea), P(eb), P(self.words))
        if self.update == "synchronous":
            lib().orc_network_update_sync(ctypes.byref(self.prog), c_int32(n), c_int32(self.updates_per_step),
                                          P(self.words))
        elif self.update == "asynchronous":
            lib().orc_network_update_async(ctypes.byref(self.prog), c_int32(n), c_int32(self.updates_per_step),
                                           P(sim.rng_state), P(self.words))
        else:
            r = self.rates
            lib().orc_network_update_maboss(ctypes.byref(self.prog), c_int32(n), f32(dt_h * self.time_units_per_h),
                                            c_int32(self.max_events), P(r["rate_up_true"]), P(r["rate_up_false"]),
                                            P(r["rate_down_true"]), P(r["rate_down_false"]), P(sim.rng_state),
                                            P(self.words))
        self.read_fates(sim)

    def inherit(self, sim: OracleSim, count_before: int) -> None:
        if count_before == 0 or sim.count == count_before:
            return
        lib().orc_network_inherit(c_int32(count_before), c_int32(self.n_words), P(sim.divide_flag),
                                  P(sim.division_offset), P(self.words))


def metabolic_update(sim: OracleSim, species: list, production_source: dict) -> list:
    """Mirror of MetabolicFields.update (fields/metabolism.py:99-111): one deposit, then per
    species in order combine -> solve (with its production source) -> sample. Returns the
    (sweeps, residual, converged) of every species."""
    n = sim.count
    geom = species[0].geom
    acc = deposit(geom, sim.position[:n], sim.cell_state[:n])
    dens, _ = density_convert(geom, acc)
    by_name = {s.name: s for s in species}
    reports = []
    for s in species:
        s.combine(dens)
        src = by_name.get(production_source.get(s.name))
        reports.append(s.solve(src.values if src is not None else None, src.michaelis_k if src is not None else 1.0))
        s.sample_into(sim, sim.local_field(s.name))
    return reports


def full_cell_step(sim: OracleSim, lifecycle, contact, dt_cells: float, dt_mechanics: float, species: list,
                   production_source: dict, network: OracleNetwork | None = None, dim: int = 128,
                   timings: dict | None = None):
    """Mirror of simulation/simulator.py:58-81 with a MetabolicFields and an optional network.

    ``timings``, when given, accumulates the seconds of each stage under "fields" (deposit, solves,
    sampling), "network", "lifecycle" (decisions, scan, placement, inheritance) and "mechanics"."""
    clock = time.perf_counter
    t0 = clock()
    reports = metabolic_update(sim, species, production_source) if species else []
    t1 = clock()
    if network is not None:
        network.step(sim, dt_cells)
    t2 = clock()
    count_before = sim.count
    sim.decide_lifecycle(lifecycle, dt_cells)
    daughters = sim.commit_divisions(lifecycle)
    if network is not None and daughters:
        network.inherit(sim, count_before)
    t3 = clock()
    substeps = max(1, int(round(dt_cells / dt_mechanics)))
    for _ in range(substeps):
        sim.contact_substep(contact.query_radius, dim, contact.query_radius, contact.rate, dt_mechanics)
    if timings is not None:
        t4 = clock()
        for stage, dt in (("fields", t1 - t0), ("network", t2 - t1), ("lifecycle", t3 - t2), ("mechanics", t4 - t3)):
            timings[stage] = timings.get(stage, 0.0) + dt
    return daughters, reports


def adjoint_forward_f64(pos0: np.ndarray, radius: np.ndarray, vmax: np.ndarray, geom: Geometry, steps: int, dt: float,
                        rate: float, query_radius: float, cell_size: float, dim: int, diffusion: float,
                        michaelis_k: float, boundary: float, omega: float = 1.8, tolerance: float = 1e-13,
                        max_sweeps: int = 200000):
    """FP64 forward of the adjoint model (exact deposit weights, double parameters): returns the
    steady field (nodes,) and the positions after ``steps`` contact steps."""
    pos = np.ascontiguousarray(pos0, dtype=np.float64).copy()
    r = np.ascontiguousarray(radius, dtype=np.float64)
    v = np.ascontiguousarray(vmax, dtype=np.float64)
    nx, ny, nz = geom.shape
    origin = np.ascontiguousarray(geom.origin, dtype=np.float64)
    field = np.zeros(geom.nodes, dtype=np.float64)
    lib().orc_adjoint_forward_f64.restype = c_int32
    sweeps = lib().orc_adjoint_forward_f64(
        c_int32(pos.shape[0]), P(pos), P(r), P(v), f32(cell_size), c_int32(dim), c_double(query_radius),
        c_double(rate), c_double(dt), c_int32(steps), c_int32(nx), c_int32(ny), c_int32(nz), P(origin),
        c_double(geom.dx), c_double(diffusion), c_double(michaelis_k), c_double(boundary), c_double(omega),
        c_double(tolerance), c_int32(max_sweeps), P(field))
    return field, pos, int(sweeps)


def contact_substep_region(pos: np.ndarray, radius: np.ndarray, cell_size: float, dim: int, query_radius: float,
                           rate: float, dt: float, region_geom: Geometry, sdf: np.ndarray, gradient: np.ndarray,
                           wall_rate: float):
    """float32 contact substep with the tissue-region push, in place on ``pos``."""
    assert pos.dtype == np.float32
    n = pos.shape[0]
    nc = np.zeros(n, dtype=np.int32)
    vel = np.zeros((n, 3), dtype=np.float32)
    r = np.ascontiguousarray(radius, dtype=np.float32)
    s = np.ascontiguousarray(sdf, dtype=np.float32)
    g = np.ascontiguousarray(gradient, dtype=np.float32)
    nx, ny, nz = region_geom.shape
    o = region_geom.origin
    lib().orc_contact_substep_region_f32(c_int32(n), P(pos), P(r), f32(cell_size), c_int32(dim), f32(query_radius),
                                         f32(rate), f32(dt), c_int32(nx), c_int32(ny), c_int32(nz), f32(o[0]),
                                         f32(o[1]), f32(o[2]), f32(1.0 / region_geom.dx), P(s), P(g), f32(wall_rate),
                                         P(vel), P(nc))
    return vel, nc


def adjoint_contact_f64(pos0: np.ndarray, radius: np.ndarray, steps: int, dt: float, rate: float, query_radius: float,
                        cell_size: float, dim: int, grad_x: np.ndarray):
    """FP64 reverse of ``steps`` contact steps from ``pos0``: (dL/dx_0, dL/drate) for dL/dx_K = grad_x."""
    pos = np.ascontiguousarray(pos0, dtype=np.float64)
    r = np.ascontiguousarray(radius, dtype=np.float64)
    lam = np.ascontiguousarray(grad_x, dtype=np.float64).copy()
    d_rate = np.zeros(1, dtype=np.float64)
    lib().orc_adjoint_contact_f64.restype = None
    lib().orc_adjoint_contact_f64(c_int32(pos.shape[0]), P(pos), P(r), f32(cell_size), c_int32(dim),
                                  c_double(query_radius), c_double(rate), c_double(dt), c_int32(steps), P(lam),
                                  P(d_rate))
    return lam, float(d_rate[0])


def contact_crossings_f64(pos0: np.ndarray, radius: np.ndarray, steps: int, dt: float, rate_a: float, rate_b: float,
                          query_radius: float, cell_size: float, dim: int) -> int:
    """Contact pairs present at a step of one FP64 trajectory (rate_a) and not of the other (rate_b)."""
    pos = np.ascontiguousarray(pos0, dtype=np.float64)
    r = np.ascontiguousarray(radius, dtype=np.float64)
    lib().orc_contact_crossings_f64.restype = ctypes.c_int64
    return int(lib().orc_contact_crossings_f64(c_int32(pos.shape[0]), P(pos), P(r), f32(cell_size), c_int32(dim),
                                               c_double(query_radius), c_double(rate_a), c_double(rate_b),
                                               c_double(dt), c_int32(steps)))


def adjoint_field_f64(pos: np.ndarray, vmax: np.ndarray, geom: Geometry, diffusion: float, michaelis_k: float,
                      u: np.ndarray, grad_u: np.ndarray, omega: float = 1.8, tolerance: float = 1e-12,
                      max_sweeps: int = 200000):
    """FP64 field half of the adjoint: ({"km", "diffusion", "boundary"}, dL/dVmax, the field's dL/dx, sweeps)."""
    p = np.ascontiguousarray(pos, dtype=np.float64)
    v = np.ascontiguousarray(vmax, dtype=np.float64)
    uu = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
    gg = np.ascontiguousarray(grad_u, dtype=np.float64).reshape(-1)
    nx, ny, nz = geom.shape
    origin = np.ascontiguousarray(geom.origin, dtype=np.float64)
    sums = np.zeros(3, dtype=np.float64)
    grad_vmax = np.zeros(p.shape[0], dtype=np.float64)
    grad_x = np.zeros_like(p)
    lib().orc_adjoint_field_f64.restype = c_int32
    sweeps = lib().orc_adjoint_field_f64(c_int32(nx), c_int32(ny), c_int32(nz), P(origin), c_double(geom.dx),
                                         c_double(diffusion), c_double(michaelis_k), c_int32(p.shape[0]), P(p), P(v),
                                         P(uu), P(gg), c_double(omega), c_double(tolerance), c_int32(max_sweeps),
                                         P(sums), P(grad_vmax), P(grad_x))
    return {"km": sums[0], "diffusion": sums[1], "boundary": sums[2]}, grad_vmax, grad_x, int(sweeps)


def adjoint_gradients_f64(pos0: np.ndarray, radius: np.ndarray, vmax: np.ndarray, geom: Geometry, steps: int,
                          dt: float, stiffness: float, damping: float, query_radius: float, cell_size: float, dim: int,
                          diffusion: float, michaelis_k: float, boundary: float, loss_grads,
                          tolerance: float = 1e-13):
    """The whole adjoint in FP64: forward (orc_adjoint_forward_f64), ``loss_grads(u, x_K) -> (dL/du,
    dL/dx_K)`` in FP64, the field adjoint, then the contact steps in reverse. Returns the gradients
    {"km", "diffusion", "boundary", "stiffness", "vmax"} of the same model the GPU adjoint differentiates."""
    rate = stiffness / damping
    field, pos, _ = adjoint_forward_f64(pos0, radius, vmax, geom, steps, dt, rate, query_radius, cell_size, dim,
                                       diffusion, michaelis_k, boundary, tolerance=tolerance)
    grad_u, grad_x = loss_grads(field, pos)
    sums, grad_vmax, field_x, _ = adjoint_field_f64(pos, vmax, geom, diffusion, michaelis_k, field, grad_u)
    _, d_rate = adjoint_contact_f64(pos0, radius, steps, dt, rate, query_radius, cell_size, dim,
                                    np.asarray(grad_x, dtype=np.float64) + field_x)
    return {**sums, "stiffness": d_rate / damping, "vmax": grad_vmax}

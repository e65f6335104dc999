"""Experiment configuration: a YAML file (or a dict) -> validated frozen dataclasses -> the model's
parameter objects (reference: simulation/config.py).

The schema is the reference's: the same sections, keys (each carrying its unit in its name),
defaults and validation rules, so its configuration files load unchanged. Unknown keys are
errors. Files are read with :mod:`yaml_subset` (PyYAML when present).
"""

from __future__ import annotations

import dataclasses
import typing
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from warpbiocell_gb300.cells.lifecycle import LifecycleParams
from warpbiocell_gb300.cells.mechanics import ContactParams
from warpbiocell_gb300.fields.diffusion import SolverSettings
from warpbiocell_gb300.fields.oxygen import OxygenParams
from warpbiocell_gb300.fields.scalar_field import GridGeometry
from warpbiocell_gb300.fields.species import SpeciesParams, by_state
from warpbiocell_gb300.simulation import yaml_subset
from warpbiocell_gb300.simulation.simulator import TimeStepping


class ConfigError(ValueError):
    pass


@dataclass(frozen=True)
class SimulationConfig:
    duration_h: float = 120.0
    dt_cells_h: float = 0.25
    dt_mechanics_h: float = 0.025
    seed: int = 0
    device: str = "auto"


@dataclass(frozen=True)
class CellsConfig:
    initial_count: int = 1000
    max_cells: int = 100_000
    radius_um: float = 8.0
    initial_spacing_factor: float = 1.0
    initial_jitter: float = 0.1


@dataclass(frozen=True)
class MechanicsConfig:
    stiffness: float = 10.0
    damping: float = 1.0
    margin_um: float = 2.0
    wall_rate_per_h: float = 10.0


@dataclass(frozen=True)
class LifecycleConfig:
    division_rate_per_h: float = 0.0289
    death_rate_per_h: float = 0.0
    anoxic_death_rate_per_h: float = 0.5
    inhibition_threshold: int = 8
    hypoxia_threshold_mmHg: float = 8.0
    death_threshold_mmHg: float = 2.0
    glucose_threshold_mM: float = 0.0
    glucose_death_threshold_mM: float = 0.0
    necrosis_requires_glucose: bool = False
    placement_factor: float = 1.0
    phenotype_model: str = "rules"
    apoptosis_rate_per_h: float = 0.0
    necrosis_rate_per_h: float = 0.0


@dataclass(frozen=True)
class GridConfig:
    box_um: float = 800.0
    dx_um: float = 20.0


@dataclass(frozen=True)
class SolverConfig:
    omega: float = 1.8
    tolerance: float = 1.0e-5
    max_sweeps: int = 2000
    check_every: int = 10


@dataclass(frozen=True)
class OxygenConfig:
    enabled: bool = True
    diffusion_um2_per_h: float = 7.2e6
    uptake_max_mmHg_um3_per_h: float = 1.4e8
    michaelis_k_mmHg: float = 3.4
    boundary_mmHg: float = 38.0
    uptake_state_factors: dict = field(default_factory=dict)
    grid: GridConfig = field(default_factory=GridConfig)
    solver: SolverConfig = field(default_factory=SolverConfig)


@dataclass(frozen=True)
class SpeciesConfig:
    """A species beyond oxygen on the oxygen grid (uptake / production per state, optional
    production source)."""

    name: str = ""
    unit: str = "mM"
    diffusion_um2_per_h: float = 2.4e5
    michaelis_k: float = 0.04
    boundary_value: float = 5.0
    uptake_max_by_state: dict = field(default_factory=dict)
    production_by_state: dict = field(default_factory=dict)
    production_source: str | None = None

    def params(self) -> SpeciesParams:
        return SpeciesParams(name=self.name, unit=self.unit, diffusion=self.diffusion_um2_per_h,
                             michaelis_k=self.michaelis_k, boundary_value=self.boundary_value,
                             uptake_max=by_state(self.uptake_max_by_state or None),
                             production=by_state(self.production_by_state or None),
                             production_source=self.production_source)


@dataclass(frozen=True)
class GeometryConfig:
    """Tissue region on the oxygen grid: sphere | ellipsoid | spheres (union) | mask."""

    enabled: bool = False
    shape: str = "sphere"
    center_um: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    radii_um: list = field(default_factory=lambda: [250.0, 200.0, 150.0])
    spheres: list = field(default_factory=list)
    mask_file: str | None = None
    mask_label: int | None = None
    mask_origin_um: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    confine: bool = True
    oxygen_source: str = "tissue_surface"
    seed_fill: bool = True
    seed_margin_um: float = 0.0
    seed_within_radius_um: float | None = None


@dataclass(frozen=True)
class NetworkInputConfig:
    node: str = ""
    source: str = "oxygen"
    threshold: float = 0.0
    above: bool = True


@dataclass(frozen=True)
class NetworkConfig:
    enabled: bool = False
    file: str = ""
    cfg: str | None = None
    update: str = "asynchronous"
    updates_per_step: int = 100
    time_units_per_h: float = 10.0
    max_events_per_step: int = 20000
    inputs: list = field(default_factory=list)
    outputs: dict = field(default_factory=dict)
    initial_states: dict = field(default_factory=dict)


@dataclass(frozen=True)
class OutputConfig:
    metrics_every_h: float = 1.0
    profile_every_h: float = 12.0
    checkpoint_every_h: float = 24.0
    shell_width_um: float = 20.0
    figures: bool = True


@dataclass(frozen=True)
class ExperimentConfig:
    name: str = "tumor_spheroid"
    simulation: SimulationConfig = field(default_factory=SimulationConfig)
    cells: CellsConfig = field(default_factory=CellsConfig)
    mechanics: MechanicsConfig = field(default_factory=MechanicsConfig)
    lifecycle: LifecycleConfig = field(default_factory=LifecycleConfig)
    oxygen: OxygenConfig = field(default_factory=OxygenConfig)
    species: list = field(default_factory=list)
    geometry: GeometryConfig = field(default_factory=GeometryConfig)
    network: NetworkConfig = field(default_factory=NetworkConfig)
    output: OutputConfig = field(default_factory=OutputConfig)

    # ---- parameter objects ------------------------------------------------------------------------
    def stepping(self) -> TimeStepping:
        return TimeStepping(dt_cells=self.simulation.dt_cells_h, dt_mechanics=self.simulation.dt_mechanics_h)

    def contact_params(self) -> ContactParams:
        m = self.mechanics
        return ContactParams(stiffness=m.stiffness, damping=m.damping, max_radius=self.cells.radius_um,
                             margin=m.margin_um, wall_rate=m.wall_rate_per_h)

    @property
    def has_glucose(self) -> bool:
        return self.oxygen.enabled and any(sp.name == "glucose" for sp in self.species)

    def lifecycle_params(self) -> LifecycleParams:
        lc, o2, glc = self.lifecycle, self.oxygen.enabled, self.has_glucose
        return LifecycleParams(
            division_rate=lc.division_rate_per_h,
            death_rate=lc.death_rate_per_h,
            anoxic_death_rate=lc.anoxic_death_rate_per_h,
            inhibition_threshold=lc.inhibition_threshold,
            hypoxia_threshold=lc.hypoxia_threshold_mmHg if o2 else 0.0,
            death_threshold=lc.death_threshold_mmHg if o2 else 0.0,
            glucose_threshold=lc.glucose_threshold_mM if glc else 0.0,
            glucose_death_threshold=lc.glucose_death_threshold_mM if glc else 0.0,
            necrosis_requires_glucose=lc.necrosis_requires_glucose and glc,
            placement_factor=lc.placement_factor,
            phenotype_model=lc.phenotype_model,
            apoptosis_rate=lc.apoptosis_rate_per_h,
            necrosis_rate=lc.necrosis_rate_per_h,
        )

    def oxygen_params(self) -> OxygenParams:
        o = self.oxygen
        return OxygenParams(diffusion_coefficient=o.diffusion_um2_per_h, uptake_max=o.uptake_max_mmHg_um3_per_h,
                            michaelis_k=o.michaelis_k_mmHg, boundary_value=o.boundary_mmHg)

    def species_params(self) -> list[SpeciesParams]:
        return [sp.params() for sp in self.species]

    def solver_settings(self) -> SolverSettings:
        s = self.oxygen.solver
        return SolverSettings(omega=s.omega, tolerance=s.tolerance, max_sweeps=s.max_sweeps,
                              check_every=s.check_every)

    def grid_geometry(self) -> GridGeometry:
        return GridGeometry.centered_cube(self.oxygen.grid.box_um, self.oxygen.grid.dx_um)

    def network_files(self, base_dir: str | Path | None = None) -> tuple[Path, Path | None]:
        n = self.network
        if not n.file:
            raise ConfigError("network.file is required when the network is enabled")
        return _resolve_path(n.file, base_dir), (_resolve_path(n.cfg, base_dir) if n.cfg else None)

    def load_network(self, base_dir: str | Path | None = None):
        from warpbiocell_gb300.network.model import load_network

        model, cfg = self.network_files(base_dir)
        return load_network(model, cfg)

    def network_params(self, base_dir: str | Path | None = None, network=None):
        from warpbiocell_gb300.network.runtime import InputClamp, NetworkParams

        n = self.network
        return NetworkParams(
            network=network or self.load_network(base_dir),
            update=n.update,
            updates_per_step=n.updates_per_step,
            time_units_per_h=n.time_units_per_h,
            max_events_per_step=n.max_events_per_step,
            inputs=tuple(InputClamp(node=i.node, source=i.source, threshold=i.threshold, above=i.above)
                         for i in n.inputs),
            outputs=dict(n.outputs) or None,
            initial_states=dict(n.initial_states),
        )

    def tissue_shape(self):
        """The analytical tissue shape (None when disabled or for a mask)."""
        from warpbiocell_gb300.geometry.shapes import Ellipsoid, Sphere, Union

        g = self.geometry
        if not g.enabled or g.shape == "mask":
            return None
        if g.shape == "sphere":
            return Sphere(center=tuple(g.center_um), radius=float(g.radii_um[0]))
        if g.shape == "ellipsoid":
            return Ellipsoid(center=tuple(g.center_um), radii=tuple(float(r) for r in g.radii_um))
        if g.shape == "spheres":
            return Union(tuple(Sphere(center=tuple(s["center_um"]), radius=float(s["radius_um"]))
                               for s in g.spheres))
        raise ConfigError(f"geometry.shape must be sphere, ellipsoid, spheres or mask, got {g.shape!r}")

    @property
    def n_steps(self) -> int:
        return int(round(self.simulation.duration_h / self.simulation.dt_cells_h))

    def to_dict(self) -> dict:
        return dataclasses.asdict(self)

    # ---- validation -------------------------------------------------------------------------------
    def validate(self, base_dir: str | Path | None = None) -> list[str]:
        """Raise ConfigError on an inconsistent configuration (ValueError from the parameter
        objects' own checks); return the warnings about a consistent but doubtful one. The rules
        and their messages follow reference simulation/config.py:331-422."""
        checks = [self._check_ranges(), self._check_parameter_objects()]
        if self.oxygen.enabled:
            checks.append(self._check_fields())
        if self.geometry.enabled:
            checks.append(self._check_geometry())
        checks += [self._check_network(base_dir), self._check_growth()]
        return [warning for check in checks for warning in check]

    def _check_ranges(self) -> list[str]:
        sim, cells, out = self.simulation, self.cells, self.output
        _require(sim.duration_h > 0.0, "simulation.duration_h must be positive")
        _require(1 <= cells.initial_count <= cells.max_cells, "cells.initial_count must be >= 1 and <= cells.max_cells")
        _require(cells.radius_um > 0.0, "cells.radius_um must be positive")
        _require(out.metrics_every_h > 0.0 and out.shell_width_um > 0.0,
                 "output intervals and shell width must be positive")
        return []

    def _check_parameter_objects(self) -> list[str]:
        # the contact law's substep bound and the lifecycle's own range checks raise ValueError
        self.contact_params().check_substep(self.simulation.dt_mechanics_h)
        self.lifecycle_params()
        return []

    def _check_fields(self) -> list[str]:
        self.oxygen_params()
        self.solver_settings()
        by_state(self.oxygen.uptake_state_factors or None, default=1.0)
        earlier = ["oxygen"]
        for sp in self.species:
            _require(bool(sp.name) and sp.name not in earlier,
                     f"species need unique, non-empty names other than 'oxygen' (got {sp.name!r})")
            _require(sp.production_source in (None, *earlier),
                     f"species {sp.name!r}: production_source must be an earlier species")
            sp.params()
            earlier.append(sp.name)
        # a random close packing (volume fraction 0.52) of the initial cells must sit inside the
        # box with one voxel to spare
        cells, box = self.cells, self.oxygen.grid.box_um
        packed = cells.radius_um * cells.initial_spacing_factor * (cells.initial_count / 0.52) ** (1.0 / 3.0)
        _require(packed + self.grid_geometry().dx <= 0.5 * box,
                 f"initial cluster radius ~{packed:.0f} um does not fit in the {box:.0f} um box with a one-voxel margin")
        warnings = []
        if self.lifecycle.necrosis_requires_glucose and not self.has_glucose:
            warnings.append("lifecycle.necrosis_requires_glucose is set but there is no species named 'glucose': "
                            "oxygen-only death applies")
        if self.lifecycle.hypoxia_threshold_mmHg >= self.oxygen.boundary_mmHg:
            warnings.append("hypoxia threshold is at or above the boundary oxygen: every cell will be hypoxic")
        return warnings

    def _check_geometry(self) -> list[str]:
        g = self.geometry
        _require(g.oxygen_source in ("tissue_surface", "box"), "geometry.oxygen_source must be tissue_surface or box")
        _require(len(g.center_um) == 3 and len(g.mask_origin_um) == 3,
                 "geometry.center_um and mask_origin_um need three components")
        if g.shape == "mask":
            _require(bool(g.mask_file), "geometry.shape = mask needs geometry.mask_file")
        else:
            _require(g.shape != "spheres" or bool(g.spheres),
                     "geometry.shape = spheres needs a non-empty geometry.spheres list")
            try:
                lower, upper = self.tissue_shape().bounds
            except ValueError as exc:
                raise ConfigError(f"geometry: {exc}") from exc
            grid = self.grid_geometry()
            inner_lo = np.asarray(grid.origin) + grid.dx
            inner_hi = np.asarray(grid.upper) - grid.dx
            _require(bool(np.all(lower >= inner_lo) and np.all(upper <= inner_hi)),
                     "the tissue shape does not fit in oxygen.grid with a one-voxel margin")
        _require(g.seed_within_radius_um is None or g.seed_within_radius_um > 0.0,
                 "geometry.seed_within_radius_um must be positive")
        return []

    def _check_network(self, base_dir) -> list[str]:
        n, model = self.network, self.lifecycle.phenotype_model
        _require(n.enabled or model != "network", "lifecycle.phenotype_model = network needs network.enabled = true")
        if not n.enabled:
            return []
        try:
            params = self.network_params(base_dir)
        except (OSError, ValueError) as exc:
            raise ConfigError(f"network: {exc}") from exc
        sources = self._network_sources()
        for clamp in params.inputs:
            _require(clamp.source in sources,
                     f"network input {clamp.node!r}: source {clamp.source!r} is not one of {sources}")
        warnings = []
        clamped = {clamp.node for clamp in params.inputs}
        p_on = {node.name: node.p_on for node in params.network.nodes}
        p_on.update(n.initial_states)
        unclamped_random = [name for name in params.network.input_names
                            if name not in clamped and 0.0 < p_on[name] < 1.0]
        if unclamped_random:
            warnings.append(f"network input nodes without a clamp are drawn once and then frozen: {unclamped_random}")
        if model == "rules":
            warnings.append("the network runs and its fate counts are recorded, but lifecycle.phenotype_model = "
                            "rules decides the phenotypes")
        else:
            _require(any(params.outputs.values()),
                     "lifecycle.phenotype_model = network needs at least one network output node")
        return warnings

    def _network_sources(self) -> list[str]:
        """What an input clamp can read: a constant, and with the fields on, oxygen, glucose and up
        to two further species (the runtime's local-value slots)."""
        if not self.oxygen.enabled:
            return ["constant"]
        names = [sp.name for sp in self.species]
        others = [name for name in names if name != "glucose"][:2]
        return ["constant", "oxygen", *(["glucose"] if "glucose" in names else []), *others]

    def _check_growth(self) -> list[str]:
        if self.lifecycle.phenotype_model != "rules":
            return []
        cells = self.cells
        unchecked = cells.initial_count * np.exp(self.lifecycle.division_rate_per_h * self.simulation.duration_h)
        if unchecked <= cells.max_cells:
            return []
        return [f"free exponential growth would reach {unchecked:.0f} cells > max_cells={cells.max_cells}; "
                "the run stops with status 'capacity_exceeded' if inhibition and death do not limit it"]


# ---- loading ------------------------------------------------------------------------------------

def _require(ok: bool, message: str) -> None:
    if not ok:
        raise ConfigError(message)


# list-valued fields whose items are themselves sections
_LIST_ITEMS = {(ExperimentConfig, "species"): SpeciesConfig, (NetworkConfig, "inputs"): NetworkInputConfig}


def _resolve_path(name, base_dir) -> Path:
    """``name`` against ``base_dir`` when it is relative and exists there (or nowhere else)."""
    path = Path(name).expanduser()
    if path.is_absolute() or base_dir is None:
        return path
    beside = Path(base_dir) / path
    return path if path.exists() and not beside.exists() else beside


def _as_bool(value, where):
    _require(isinstance(value, bool), f"{where}: expected true/false, got {value!r}")
    return value


def _as_int(value, where):
    integral = isinstance(value, (int, float)) and not isinstance(value, bool) and float(value).is_integer()
    _require(integral, f"{where}: expected an integer, got {value!r}")
    return int(value)


def _as_float(value, where):
    if isinstance(value, str):  # YAML 1.1 reads 1e-5 (no dot) as a string
        try:
            return float(value)
        except ValueError:
            raise ConfigError(f"{where}: expected a number, got {value!r}") from None
    _require(isinstance(value, (int, float)) and not isinstance(value, bool),
             f"{where}: expected a number, got {value!r}")
    return float(value)


def _as_str(value, where):
    _require(isinstance(value, str), f"{where}: expected a string, got {value!r}")
    return value


# declared type -> conversion; other annotations (dicts, lists, optionals) pass values through
_SCALARS = {bool: _as_bool, int: _as_int, float: _as_float, str: _as_str}


def _convert(owner, key, declared, value, where):
    if dataclasses.is_dataclass(declared):
        return _build(declared, value, where)
    item = _LIST_ITEMS.get((owner, key))
    if item is not None:
        _require(isinstance(value, list), f"{where} must be a list")
        return [_build(item, entry, f"{where}[{i}]") for i, entry in enumerate(value)]
    convert = _SCALARS.get(declared)
    return value if convert is None else convert(value, where)


def _build(cls, data, where: str):
    """The dataclass ``cls`` from a mapping; ``where`` names it in errors (``config.oxygen`` ...)."""
    _require(isinstance(data, dict), f"{where}: expected a mapping, got {type(data).__name__}")
    declared = typing.get_type_hints(cls)
    valid = sorted(f.name for f in dataclasses.fields(cls))
    unknown = sorted(key for key in data if key not in valid)
    _require(not unknown, f"{where}: unknown keys {unknown}; valid keys are {valid}")
    values = {key: _convert(cls, key, declared[key], value, f"{where}.{key}") for key, value in data.items()}
    try:
        return cls(**values)
    except TypeError as exc:
        raise ConfigError(f"{where}: {exc}") from exc


def config_from_dict(data: dict) -> ExperimentConfig:
    return _build(ExperimentConfig, data or {}, "config")


def apply_overrides(data: dict, overrides: list[str]) -> dict:
    """Apply ``section.key=value`` overrides (values read as YAML scalars) to a nested dict, in
    place, creating missing sections."""
    for item in overrides:
        dotted, equals, text = item.partition("=")
        _require(bool(equals), f"override {item!r} must look like section.key=value")
        *sections, leaf = dotted.strip().split(".")
        target = data
        for name in sections:
            target = target.setdefault(name, {})
            _require(isinstance(target, dict), f"override {item!r}: {name} is not a section")
        try:
            target[leaf] = yaml_subset.scalar(text)
        except ValueError as exc:
            raise ConfigError(f"override {item!r}: {exc}") from exc
    return data


def resolve_file_references(data: dict, base_dir: str | Path) -> dict:
    """Make the network model and .cfg names absolute against ``base_dir`` where they exist there."""
    network = data.get("network")
    if not isinstance(network, dict):
        return data
    for key in ("file", "cfg"):
        name = network.get(key)
        if isinstance(name, str) and name:
            network[key] = str(_resolve_path(name, base_dir))
    return data


def read_yaml(path: str | Path) -> dict:
    try:
        return yaml_subset.safe_load(Path(path).read_text()) or {}
    except ValueError as exc:
        raise ConfigError(f"{path}: {exc}") from exc


def load_config(path: str | Path, overrides: list[str] | None = None) -> ExperimentConfig:
    path = Path(path)
    data = read_yaml(path)
    if overrides:
        apply_overrides(data, overrides)
    resolve_file_references(data, path.parent)
    return config_from_dict(data)

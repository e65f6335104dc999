"""Experiment: build every model object from a configuration, run it, record everything
(reference: simulation/experiment.py).

    experiment = Experiment(config)
    result = experiment.run(output_dir)      # or run() for an in-memory result
    result.metrics[-1]["living_cells"]

The step loop is the plain cell step on one GPU; the host synchronises only where the reference
does (metrics, profiles and checkpoints at their intervals, and the division count inside each
step). :meth:`Experiment.resume` continues a run from one of its checkpoints bit for bit.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field
from pathlib import Path
from typing import Callable

import numpy as np
import torch

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.cells.initialization import spherical_cluster
from warpbiocell_gb300.cells.lifecycle import CapacityError
from warpbiocell_gb300.cells.mechanics import contact_substep, make_neighbor_grid
from warpbiocell_gb300.cells.state import CellPopulation
from warpbiocell_gb300.fields.metabolism import MetabolicFields
from warpbiocell_gb300.fields.oxygen import OxygenField
from warpbiocell_gb300.geometry.region import TissueRegion
from warpbiocell_gb300.geometry.seeding import fill_region
from warpbiocell_gb300.geometry.shapes import Sphere
from warpbiocell_gb300.io.checkpoints import (load_checkpoint, restore_fields, restore_network, restore_population,
                                             save_checkpoint)
from warpbiocell_gb300.io.run_output import RunOutput
from warpbiocell_gb300.metrics.population import population_summary, radial_profile, shell_radii
from warpbiocell_gb300.simulation.config import ExperimentConfig
from warpbiocell_gb300.simulation.simulator import cell_step


@dataclass
class RunResult:
    status: str  # "completed" | "capacity_exceeded"
    metrics: list[dict] = field(default_factory=list)
    profiles: list[tuple[float, dict]] = field(default_factory=list)
    summary: dict | None = None
    output_dir: Path | None = None
    wall_s: float = 0.0

    def metric(self, name: str) -> np.ndarray:
        return np.array([row[name] for row in self.metrics], dtype=float)


# metrics column -> population_summary key, for the columns copied as they are
_SUMMARY_COLUMNS = {
    "cells": "cells", "living_cells": "living_cells", "dead_cells": "dead_cells",
    "proliferative_cells": "proliferative_cells", "quiescent_cells": "quiescent_cells",
    "hypoxic_cells": "hypoxic_cells", "mean_radius_um": "mean_radius", "spheroid_radius_um": "spheroid_radius",
}
# metrics column -> population_summary key of a field statistic, NaN when the run has no such field
_FIELD_COLUMNS = {
    "oxygen_cells_mean_mmHg": "oxygen_cells_mean", "oxygen_cells_min_mmHg": "oxygen_cells_min",
    "oxygen_grid_mean_mmHg": "oxygen_grid_mean", "oxygen_grid_min_mmHg": "oxygen_grid_min",
    "glucose_cells_mean_mM": "glucose_cells_mean", "glucose_cells_min_mM": "glucose_cells_min",
    "lactate_cells_mean_mM": "lactate_cells_mean", "lactate_cells_max_mM": "lactate_cells_max",
}
_FATE_ROLES = ("proliferation", "apoptosis", "growth_arrest", "necrosis")


def _cells_outside(population, oxygen, region) -> tuple[int, int]:
    """Cells outside the field's grid and outside the tissue region (0 where there is none)."""
    if oxygen is None and region is None:
        return 0, 0
    positions = population.positions_numpy()
    grid = 0 if oxygen is None else int(np.count_nonzero(~oxygen.geometry.contains(positions)))
    tissue = 0 if region is None else int(np.count_nonzero(~region.contains(positions)))
    return grid, tissue


def observe(population, oxygen, time_h: float, shell_width: float = 20.0, region=None, network=None,
            wall_s: float = 0.0, field_sweeps: int = 0) -> tuple[dict, dict]:
    """The metrics row of a population (the columns of ``io.run_output.METRIC_COLUMNS``) and the
    radial profile it was derived from; ``oxygen`` is an OxygenField or MetabolicFields (or None),
    ``region`` a TissueRegion, ``network`` a NetworkRuntime (reference:
    simulation/experiment.py:50-98). A rim is the spheroid radius less the radius of the
    necrotic (non-proliferative) core, floored at zero; network fate counts are empty without a
    network."""
    summary = population_summary(population, oxygen)
    profile = radial_profile(population, shell_width=shell_width)
    radii = shell_radii(profile)
    outside_grid, outside_tissue = _cells_outside(population, oxygen, region)
    outer = summary["spheroid_radius"]
    row = {"time_h": time_h}
    row.update({column: summary[key] for column, key in _SUMMARY_COLUMNS.items()})
    row.update({f"{key}_um": radii[key] for key in ("necrotic_radius", "hypoxic_radius", "non_proliferative_radius")})
    row["viable_rim_um"] = max(0.0, outer - radii["necrotic_radius"])
    row["proliferating_rim_um"] = max(0.0, outer - radii["non_proliferative_radius"])
    row.update({column: summary.get(key, float("nan")) for column, key in _FIELD_COLUMNS.items()})
    fates = {} if network is None else network.fate_counts(population)
    row.update({f"network_{role}_cells": fates.get(role, "") for role in _FATE_ROLES})
    row.update(field_sweeps=field_sweeps, cells_outside_grid=outside_grid, cells_outside_tissue=outside_tissue,
               wall_s=wall_s)
    return row, profile


def _resolve_device(name):
    return _lib.resolve_device(None if name in (None, "auto") else name)


@dataclass
class _Schedule:
    """Which outputs fall due after a step: every interval in steps, and all of them at the last."""

    metrics: int
    profile: int
    checkpoint: int
    last: int

    @classmethod
    def of(cls, output, dt_h: float, n_steps: int) -> "_Schedule":
        def steps(hours):
            return max(1, int(round(hours / dt_h)))

        return cls(steps(output.metrics_every_h), steps(output.profile_every_h), steps(output.checkpoint_every_h),
                   n_steps)

    def due(self, step: int) -> tuple[bool, bool, bool]:
        final = step == self.last
        return tuple(final or step % every == 0 for every in (self.metrics, self.profile, self.checkpoint))


class _Recorder:
    """Sends each observation to the in-memory result, the run directory and the callbacks."""

    def __init__(self, experiment: "Experiment", result: RunResult, output: RunOutput | None,
                 log: Callable[[str], None] | None, on_metrics: Callable[[dict], None] | None):
        self.experiment, self.result, self.output = experiment, result, output
        self.log = log or (lambda message: None)
        self.on_metrics = on_metrics

    def __call__(self, wall: float, sweeps: int, metrics=True, profile=True, checkpoint=True) -> dict:
        exp = self.experiment
        row, prof = exp.observe(wall, sweeps)
        if metrics:
            self.result.metrics.append(row)
            if self.output:
                self.output.write_metrics(row)
            if self.on_metrics:
                self.on_metrics(row)
            self.log(f"t={exp.time_h:7.2f} h  cells={row['cells']:7d}  prolif={row['proliferative_cells']:6d}  "
                     f"hypoxic={row['hypoxic_cells']:6d}  dead={row['dead_cells']:6d}  "
                     f"R={row['spheroid_radius_um']:6.1f} um  O2min={row['oxygen_cells_min_mmHg']:6.2f}  "
                     f"wall={wall:7.1f} s")
            if row["cells_outside_grid"]:
                self.log(f"warning: {row['cells_outside_grid']} cells lie outside the oxygen grid and are ignored "
                         "by the field")
        if profile:
            self.result.profiles.append((exp.time_h, prof))
            if self.output:
                self.output.write_profile(exp.time_h, prof)
        if checkpoint and self.output:
            exp.save(self.output.checkpoint_path(exp.time_h))
        return row


class Experiment:
    """Every model object of one configuration, the state they evolve, and the run loop
    (reference: simulation/experiment.py:101-246)."""

    def __init__(self, config: ExperimentConfig, device: str | None = None, config_path: str | Path | None = None):
        self.config = config
        self.config_path = Path(config_path) if config_path else None
        self.base_dir = self.config_path.parent if self.config_path else None
        self.warnings = config.validate(self.base_dir)
        self.device = _resolve_device(device or config.simulation.device)
        self.region = self._build_region() if config.geometry.enabled else None
        self.population = self._seed_population()
        self.contact = config.contact_params()
        self.grid = make_neighbor_grid(self.contact, self.device)
        self.lifecycle = config.lifecycle_params()
        self.stepping = config.stepping()
        self.oxygen = self._build_fields() if config.oxygen.enabled else None
        self.confine = self.region if config.geometry.confine else None
        self.network = self._build_network() if config.network.enabled else None
        self.time_h = 0.0
        self._resumed_step = 0

    # ---- construction ----------------------------------------------------------------------------
    def _build_region(self) -> TissueRegion:
        g = self.config.geometry
        if g.shape == "mask":  # reference: simulation/experiment.py:141-145
            from warpbiocell_gb300.geometry.masks import load_nifti_mask, region_from_mask
            from warpbiocell_gb300.simulation.config import _resolve_path

            path = _resolve_path(g.mask_file, self.base_dir)
            mask, voxel = load_nifti_mask(path, g.mask_label)
            return region_from_mask(mask, voxel, self.config.grid_geometry(), mask_origin=tuple(g.mask_origin_um),
                                    device=self.device, name=Path(g.mask_file).name)
        return TissueRegion.from_shape(self.config.tissue_shape(), self.config.grid_geometry(), device=self.device)

    def _seed_population(self) -> CellPopulation:
        cells = self.config.cells
        positions = self._initial_positions()
        radii = np.full(positions.shape[0], cells.radius_um)
        return CellPopulation.from_numpy(positions, radii, capacity=cells.max_cells, device=self.device,
                                         seed=self.config.simulation.seed)

    def _initial_positions(self) -> np.ndarray:
        """A filled tissue region, or a packed cluster (moved to the region's centre when there is
        one, with a warning for cells that land outside it)."""
        cfg = self.config
        cells, g = cfg.cells, cfg.geometry
        packing = dict(spacing_factor=cells.initial_spacing_factor, jitter=cells.initial_jitter,
                       seed=cfg.simulation.seed)
        if self.region is not None and g.seed_fill:
            within = None
            if g.seed_within_radius_um:
                within = Sphere(center=tuple(g.center_um), radius=g.seed_within_radius_um)
            return fill_region(self.region, cells.radius_um, margin=g.seed_margin_um, max_cells=cells.max_cells,
                               within=within, **packing)
        positions = spherical_cluster(cells.initial_count, cells.radius_um, **packing)
        if self.region is None:
            return positions
        positions += np.asarray(g.center_um, dtype=np.float32)
        stray = int(np.count_nonzero(~self.region.contains(positions, margin=cells.radius_um)))
        if stray:
            self.warnings.append(f"{stray} of the {positions.shape[0]} initial cells lie outside the tissue region")
        return positions

    def _build_fields(self):
        """OxygenField alone, or MetabolicFields when the run has more species or per-state uptake;
        the tissue boundary holds the supply when the region is the oxygen source."""
        cfg = self.config
        fixed_outside = self.region if cfg.geometry.oxygen_source == "tissue_surface" else None
        common = dict(device=self.device, fixed_outside=fixed_outside)
        if cfg.species or cfg.oxygen.uptake_state_factors:
            return MetabolicFields(cfg.grid_geometry(), cfg.oxygen_params(), cfg.species_params(),
                                   cfg.solver_settings(), oxygen_state_factors=cfg.oxygen.uptake_state_factors or None,
                                   **common)
        return OxygenField(cfg.grid_geometry(), cfg.oxygen_params(), cfg.solver_settings(), **common)

    def _build_network(self):
        from warpbiocell_gb300.network.runtime import NetworkRuntime

        cfg = self.config
        species = ("oxygen", *(sp.name for sp in cfg.species)) if cfg.oxygen.enabled else ()
        runtime = NetworkRuntime(cfg.network_params(self.base_dir), capacity=cfg.cells.max_cells, device=self.device,
                                 species_names=species)
        runtime.initialize(self.population)
        return runtime

    # ---- checkpoints -----------------------------------------------------------------------------
    def save(self, path: str | Path) -> Path:
        return save_checkpoint(path, self.population, self.oxygen, self.time_h, region=self.region,
                               network=self.network)

    def resume(self, checkpoint: str | Path | dict) -> None:
        """Replace the state by a checkpoint of this configuration's run; :meth:`run` then continues
        from the checkpoint's time and gives the bits the uninterrupted run would have given."""
        data = checkpoint if isinstance(checkpoint, dict) else load_checkpoint(checkpoint)
        if int(data["seed"]) != self.config.simulation.seed:
            raise ValueError("the checkpoint was written with another seed")
        self.population = restore_population(data, capacity=self.config.cells.max_cells, device=self.device)
        if self.oxygen is not None:
            restore_fields(data, self.oxygen)
        if self.network is not None:
            restore_network(data, self.network, self.population)
        self.time_h = float(data["time_h"])
        self._resumed_step = int(round(self.time_h / self.stepping.dt_cells))

    # ---- observation -----------------------------------------------------------------------------
    def observe(self, wall_s: float = 0.0, field_sweeps: int = 0) -> tuple[dict, dict]:
        return observe(self.population, self.oxygen, self.time_h, shell_width=self.config.output.shell_width_um,
                       region=self.region, network=self.network, wall_s=wall_s, field_sweeps=field_sweeps)

    def _synchronize(self) -> None:
        torch.cuda.synchronize(self.device)

    # ---- run -------------------------------------------------------------------------------------
    def _open_output(self, output_dir) -> RunOutput:
        cfg = self.config
        output = RunOutput(Path(output_dir), self.config_path, cfg.to_dict(), self.device, cfg.simulation.seed)
        meta = output.metadata
        meta["warnings"] = list(self.warnings)
        if self.region is not None:
            meta["tissue"] = {"name": self.region.name, "volume_um3": self.region.volume(),
                              "seeded_cells": self.population.count, "confined": self.confine is not None,
                              "oxygen_source": cfg.geometry.oxygen_source}
        if self.network is not None:
            net = self.network.network
            meta["network"] = {"source": net.source, "nodes": net.n_nodes, "inputs": net.input_names,
                               "update": cfg.network.update, "phenotype_model": cfg.lifecycle.phenotype_model}
        if self._resumed_step:
            meta["resumed_from_h"] = self.time_h
        output.write_metadata()
        return output

    def _prime(self) -> None:
        """Neighbour counts, fields and network inputs of the initial state (a fresh run only)."""
        contact_substep(self.population, self.grid, self.contact, dt=0.0)
        if self.oxygen is not None:
            self.oxygen.update(self.population)
        if self.network is not None:
            self.network.clamp_inputs(self.population)
            self.network.read_fates(self.population)

    def run(self, output_dir: str | Path | None = None, log: Callable[[str], None] | None = None,
            on_metrics: Callable[[dict], None] | None = None) -> RunResult:
        """Run to the end. ``log`` receives human-readable lines, ``on_metrics`` every metrics row.
        A population that outgrows its capacity ends the run early with the status
        ``capacity_exceeded`` and a final observation of the state it reached."""
        cfg = self.config
        dt_h = self.stepping.dt_cells
        schedule = _Schedule.of(cfg.output, dt_h, cfg.n_steps)
        output = self._open_output(output_dir) if output_dir is not None else None
        result = RunResult(status="completed", output_dir=Path(output_dir) if output_dir else None)
        record = _Recorder(self, result, output, log, on_metrics)
        for message in self.warnings:
            record.log(f"warning: {message}")
        if not self._resumed_step:
            self._prime()

        t0 = time.perf_counter()
        last_row = record(0.0, 0, checkpoint=not self._resumed_step)
        sweeps = 0
        for step in range(self._resumed_step + 1, cfg.n_steps + 1):
            try:
                report = cell_step(self.population, self.grid, self.lifecycle, self.contact, self.stepping,
                                   oxygen=self.oxygen, region=self.confine, network=self.network)
            except CapacityError as exc:
                result.status = "capacity_exceeded"
                record.log(f"stopping: {exc}")
                break
            sweeps = report.field_sweeps
            self.time_h = step * dt_h
            if not report.field_converged:
                record.log(f"warning: field solve reached max_sweeps at t={self.time_h:.2f} h "
                           f"(residual {report.field_residual:.2e})")
            due = schedule.due(step)
            if any(due):
                self._synchronize()
                row = record(time.perf_counter() - t0, sweeps, *due)
                if due[0]:
                    last_row = row
        self._synchronize()
        result.wall_s = time.perf_counter() - t0
        if result.status != "completed":
            last_row = record(result.wall_s, sweeps)
        result.summary = {**last_row, "steps": int(round(self.time_h / dt_h)), "status": result.status}
        if output:
            if cfg.output.figures:
                record.log("figures skipped: no plotting backend in this package")
            output.finish(result.status, result.wall_s, result.summary)
        return result

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


def observe(population, oxygen, time_h: float, shell_width: float = 20.0, region=None, network=None,
            wall_s: float = 0.0, field_sweeps: int = 0) -> tuple[dict, dict]:
    """The metrics row of a population (the columns of ``io.run_output.METRIC_COLUMNS``) and the
    radial profile it was derived from; ``oxygen`` is an OxygenField or MetabolicFields (or None),
    ``region`` a TissueRegion, ``network`` a NetworkRuntime."""
    summary = population_summary(population, oxygen)
    profile = radial_profile(population, shell_width=shell_width)
    radii = shell_radii(profile)
    outside = outside_tissue = 0
    if oxygen is not None or region is not None:
        positions = population.positions_numpy()
        if oxygen is not None:
            outside = int((~oxygen.geometry.contains(positions)).sum())
        if region is not None:
            outside_tissue = int((~region.contains(positions)).sum())
    nan = float("nan")
    row = {
        "time_h": time_h,
        "cells": summary["cells"],
        "living_cells": summary["living_cells"],
        "dead_cells": summary["dead_cells"],
        "proliferative_cells": summary["proliferative_cells"],
        "quiescent_cells": summary["quiescent_cells"],
        "hypoxic_cells": summary["hypoxic_cells"],
        "mean_radius_um": summary["mean_radius"],
        "spheroid_radius_um": summary["spheroid_radius"],
        "necrotic_radius_um": radii["necrotic_radius"],
        "hypoxic_radius_um": radii["hypoxic_radius"],
        "non_proliferative_radius_um": radii["non_proliferative_radius"],
        "viable_rim_um": max(0.0, summary["spheroid_radius"] - radii["necrotic_radius"]),
        "proliferating_rim_um": max(0.0, summary["spheroid_radius"] - radii["non_proliferative_radius"]),
        "oxygen_cells_mean_mmHg": summary.get("oxygen_cells_mean", nan),
        "oxygen_cells_min_mmHg": summary.get("oxygen_cells_min", nan),
        "oxygen_grid_mean_mmHg": summary.get("oxygen_grid_mean", nan),
        "oxygen_grid_min_mmHg": summary.get("oxygen_grid_min", nan),
        "glucose_cells_mean_mM": summary.get("glucose_cells_mean", nan),
        "glucose_cells_min_mM": summary.get("glucose_cells_min", nan),
        "lactate_cells_mean_mM": summary.get("lactate_cells_mean", nan),
        "lactate_cells_max_mM": summary.get("lactate_cells_max", nan),
        "field_sweeps": field_sweeps,
        "cells_outside_grid": outside,
        "cells_outside_tissue": outside_tissue,
        "wall_s": wall_s,
    }
    fates = network.fate_counts(population) if network is not None else {}
    for role in ("proliferation", "apoptosis", "growth_arrest", "necrosis"):
        row[f"network_{role}_cells"] = fates.get(role, "")
    return row, profile


def _resolve_device(name):
    if name in (None, "auto"):
        return _lib.resolve_device(None)
    return _lib.resolve_device(name)


class Experiment:
    def __init__(self, config: ExperimentConfig, device: str | None = None, config_path: str | Path | None = None):
        self.config = config
        self.config_path = Path(config_path) if config_path else None
        self.base_dir = self.config_path.parent if self.config_path else None
        self.warnings = config.validate(self.base_dir)
        self.device = _resolve_device(device or config.simulation.device)

        cells = config.cells
        self.region = self._build_region() if config.geometry.enabled else None
        positions = self._initial_positions()
        self.population = CellPopulation.from_numpy(positions, np.full(positions.shape[0], cells.radius_um),
                                                    capacity=cells.max_cells, device=self.device,
                                                    seed=config.simulation.seed)
        self.contact = config.contact_params()
        self.grid = make_neighbor_grid(self.contact, self.device)
        self.lifecycle = config.lifecycle_params()
        self.stepping = config.stepping()
        fixed_outside = self.region if (self.region is not None and
                                        config.geometry.oxygen_source == "tissue_surface") else None
        self.oxygen = None
        if config.oxygen.enabled:
            if config.species or config.oxygen.uptake_state_factors:
                self.oxygen = MetabolicFields(config.grid_geometry(), config.oxygen_params(), config.species_params(),
                                              config.solver_settings(), device=self.device,
                                              fixed_outside=fixed_outside,
                                              oxygen_state_factors=config.oxygen.uptake_state_factors or None)
            else:
                self.oxygen = OxygenField(config.grid_geometry(), config.oxygen_params(), config.solver_settings(),
                                          device=self.device, fixed_outside=fixed_outside)
        self.confine = self.region if (self.region is not None and config.geometry.confine) else None
        self.network = None
        if config.network.enabled:
            from warpbiocell_gb300.network.runtime import NetworkRuntime

            species_names = ("oxygen", *(sp.name for sp in config.species)) if config.oxygen.enabled else ()
            self.network = NetworkRuntime(config.network_params(self.base_dir), capacity=cells.max_cells,
                                          device=self.device, species_names=species_names)
            self.network.initialize(self.population)
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

    def _initial_positions(self) -> np.ndarray:
        cfg = self.config
        cells, g, seed = cfg.cells, cfg.geometry, cfg.simulation.seed
        if self.region is not None and g.seed_fill:
            within = Sphere(center=tuple(g.center_um), radius=g.seed_within_radius_um) if g.seed_within_radius_um \
                else None
            return fill_region(self.region, cells.radius_um, spacing_factor=cells.initial_spacing_factor,
                               jitter=cells.initial_jitter, seed=seed, margin=g.seed_margin_um,
                               max_cells=cells.max_cells, within=within)
        positions = spherical_cluster(cells.initial_count, cells.radius_um, spacing_factor=cells.initial_spacing_factor,
                                      jitter=cells.initial_jitter, seed=seed)
        if self.region is not None:
            positions += np.asarray(g.center_um, dtype=np.float32)
            outside = int((~self.region.contains(positions, margin=cells.radius_um)).sum())
            if outside:
                self.warnings.append(f"{outside} of the {positions.shape[0]} initial cells lie outside the tissue region")
        return positions

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
    def run(self, output_dir: str | Path | None = None, log: Callable[[str], None] | None = None,
            on_metrics: Callable[[dict], None] | None = None) -> RunResult:
        """Run to the end. ``log`` receives human-readable lines, ``on_metrics`` every metrics row."""
        cfg = self.config
        out = cfg.output
        stepping = self.stepping

        def every(hours):
            return max(1, int(round(hours / stepping.dt_cells)))

        metrics_every, profile_every, checkpoint_every = (every(out.metrics_every_h), every(out.profile_every_h),
                                                          every(out.checkpoint_every_h))
        output = None
        if output_dir is not None:
            output = RunOutput(Path(output_dir), self.config_path, cfg.to_dict(), self.device, cfg.simulation.seed)
            output.metadata["warnings"] = list(self.warnings)
            if self.region is not None:
                output.metadata["tissue"] = {"name": self.region.name, "volume_um3": self.region.volume(),
                                             "seeded_cells": self.population.count,
                                             "confined": self.confine is not None,
                                             "oxygen_source": cfg.geometry.oxygen_source}
            if self.network is not None:
                net = self.network.network
                output.metadata["network"] = {"source": net.source, "nodes": net.n_nodes, "inputs": net.input_names,
                                              "update": cfg.network.update,
                                              "phenotype_model": cfg.lifecycle.phenotype_model}
            if self._resumed_step:
                output.metadata["resumed_from_h"] = self.time_h
            output.write_metadata()
        for message in self.warnings:
            if log:
                log(f"warning: {message}")

        result = RunResult(status="completed", output_dir=Path(output_dir) if output_dir else None)
        if not self._resumed_step:
            contact_substep(self.population, self.grid, self.contact, dt=0.0)  # initial neighbour counts
            if self.oxygen is not None:
                self.oxygen.update(self.population)
            if self.network is not None:
                self.network.clamp_inputs(self.population)
                self.network.read_fates(self.population)

        def record(wall, sweeps, metrics=True, profile=True, checkpoint=True):
            row, prof = self.observe(wall, sweeps)
            if metrics:
                result.metrics.append(row)
                if output:
                    output.write_metrics(row)
                if on_metrics:
                    on_metrics(row)
                if log:
                    log(f"t={self.time_h:7.2f} h  cells={row['cells']:7d}  prolif={row['proliferative_cells']:6d}  "
                        f"hypoxic={row['hypoxic_cells']:6d}  dead={row['dead_cells']:6d}  "
                        f"R={row['spheroid_radius_um']:6.1f} um  O2min={row['oxygen_cells_min_mmHg']:6.2f}  "
                        f"wall={wall:7.1f} s")
                    if row["cells_outside_grid"]:
                        log(f"warning: {row['cells_outside_grid']} cells lie outside the oxygen grid and are ignored "
                            "by the field")
            if profile:
                result.profiles.append((self.time_h, prof))
                if output:
                    output.write_profile(self.time_h, prof)
            if checkpoint and output:
                self.save(output.checkpoint_path(self.time_h))
            return row

        t_start = time.perf_counter()
        record(0.0, 0, checkpoint=not self._resumed_step)
        n_steps = cfg.n_steps
        status = "completed"
        sweeps = 0
        wall = 0.0
        last_row = result.metrics[-1]
        for step in range(self._resumed_step + 1, n_steps + 1):
            try:
                report = cell_step(self.population, self.grid, self.lifecycle, self.contact, stepping,
                                   oxygen=self.oxygen, region=self.confine, network=self.network)
            except CapacityError as exc:
                status = "capacity_exceeded"
                if log:
                    log(f"stopping: {exc}")
                break
            sweeps = report.field_sweeps
            self.time_h = step * stepping.dt_cells
            if not report.field_converged and log:
                log(f"warning: field solve reached max_sweeps at t={self.time_h:.2f} h "
                    f"(residual {report.field_residual:.2e})")
            last = step == n_steps
            due = (step % metrics_every == 0 or last, step % profile_every == 0 or last,
                   step % checkpoint_every == 0 or last)
            if any(due):
                self._synchronize()
                wall = time.perf_counter() - t_start
                row = record(wall, sweeps, *due)
                if due[0]:
                    last_row = row
        self._synchronize()
        wall = time.perf_counter() - t_start
        if status != "completed":
            last_row = record(wall, sweeps)
        result.status = status
        result.wall_s = wall
        result.summary = {**last_row, "steps": int(round(self.time_h / stepping.dt_cells)), "status": status}
        if output:
            if out.figures and log:
                log("figures skipped: no plotting backend in this package")
            output.finish(status, wall, result.summary)
        return result

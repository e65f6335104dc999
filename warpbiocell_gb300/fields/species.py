"""A diffusible species with per-state uptake and production, solved on a ScalarField
(reference: fields/species.py:35-195).

Per cell state k: ``uptake_max[k]`` (Michaelis-Menten uptake) and ``production[k]`` (zero-order,
optionally scaled by S/(K_S + S) of a source species). The per-state densities are deposited
once per step and combined into this species' consuming density and production capacity.
``update`` = deposit (if owner) -> combine -> solve -> sample, the per-cell-step sequence; when
the species owns its densities and does not produce, deposit conversion and combination are
one fused pass (``wbc_density_convert`` with weights).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from warpbiocell_gb300 import _lib, profiling
from warpbiocell_gb300.cells.model import NUM_STATES, CellState
from warpbiocell_gb300.fields.densities import CellDensities
from warpbiocell_gb300.fields.diffusion import (
    SolveReport,
    SolverSettings,
    UptakeKinetics,
    explicit_step,
    solve_steady_state,
)
from warpbiocell_gb300.fields.scalar_field import Boundary, GridGeometry, ScalarField


def by_state(values: dict | float | None, default: float = 0.0) -> tuple[float, float, float, float]:
    """Per-state tuple from a scalar (living states only), a mapping keyed by state name, or None."""
    if values is None:
        return (default,) * NUM_STATES
    if isinstance(values, (int, float)):
        return (float(values),) * (NUM_STATES - 1) + (0.0,)
    out = [default] * NUM_STATES
    for key, value in values.items():
        out[int(CellState[str(key).upper()])] = float(value)
    return tuple(out)


@dataclass(frozen=True)
class SpeciesParams:
    name: str
    unit: str
    diffusion: float
    michaelis_k: float
    boundary_value: float
    uptake_max: tuple[float, float, float, float] = (0.0, 0.0, 0.0, 0.0)
    production: tuple[float, float, float, float] = (0.0, 0.0, 0.0, 0.0)
    production_source: str | None = None
    extra: dict = field(default_factory=dict)

    def __post_init__(self):
        if not self.name:
            raise ValueError("species needs a name")
        if len(self.uptake_max) != NUM_STATES or len(self.production) != NUM_STATES:
            raise ValueError(f"uptake_max and production need {NUM_STATES} per-state values")
        if min(self.uptake_max) < 0.0 or min(self.production) < 0.0:
            raise ValueError("rates must be non-negative")
        if self.boundary_value < 0.0:
            raise ValueError("boundary_value must be non-negative")
        UptakeKinetics(self.diffusion, max(self.uptake_max), self.michaelis_k)

    @property
    def uptake_scale(self) -> float:
        return max(self.uptake_max) if self.consumes else 0.0

    @property
    def uptake_weights(self) -> tuple[float, ...]:
        scale = self.uptake_scale
        return tuple(u / scale if scale > 0.0 else 0.0 for u in self.uptake_max)

    @property
    def kinetics(self) -> UptakeKinetics:
        return UptakeKinetics(self.diffusion, self.uptake_scale, self.michaelis_k)

    @property
    def consumes(self) -> bool:
        return max(self.uptake_max) > 0.0

    @property
    def produces(self) -> bool:
        return max(self.production) > 0.0


class SpeciesField:
    """One species: its ScalarField, effective density, production capacity and solver buffers."""

    def __init__(self, geometry: GridGeometry, params: SpeciesParams, settings: SolverSettings = SolverSettings(),
                 boundary: tuple[Boundary, Boundary, Boundary] = (Boundary.DIRICHLET,) * 3, device=None,
                 fixed_outside=None, densities: CellDensities | None = None):
        self.species = params
        self.settings = settings
        self.field = ScalarField.create(geometry, params.boundary_value, boundary=boundary, device=device)
        self.device = self.field.device
        if fixed_outside is not None:
            if tuple(fixed_outside.geometry.shape) != tuple(geometry.shape):
                raise ValueError("the tissue region must be defined on the field grid")
            self.field.set_fixed(~fixed_outside.inside_mask())
        self.densities = densities if densities is not None else CellDensities(geometry, device=self.device)
        self.owns_densities = densities is None
        self.density = torch.zeros(geometry.shape, dtype=torch.float32, device=self.device)
        self.production = torch.zeros(geometry.shape, dtype=torch.float32, device=self.device)
        self._scratch = torch.zeros(geometry.shape, dtype=torch.float32, device=self.device)
        self._residual = torch.zeros(1, dtype=torch.float32, device=self.device)
        self.last_report: SolveReport | None = None

    @property
    def params(self) -> SpeciesParams:
        return self.species

    @property
    def name(self) -> str:
        return self.species.name

    @property
    def geometry(self) -> GridGeometry:
        return self.field.geometry

    @property
    def values(self) -> torch.Tensor:
        return self.field.values

    def numpy(self) -> np.ndarray:
        return self.field.numpy()

    # ---- cell <-> field transfer -------------------------------------------------------------
    def deposit_uptake(self, population) -> None:
        """Deposit the per-state densities (when this species owns them) and combine them."""
        if self.owns_densities:
            self.densities.deposit_fixed_point(population)
            if self.species.produces:
                # per-state densities and this species' consuming density in one pass, then production
                self.densities.convert(self.species.uptake_weights, self.density)
                self.densities.combine(self.species.production, self.production)
            else:
                # only the consuming density; the per-state densities when someone reads them
                self.densities.convert_combined(self.species.uptake_weights, self.density)
            return
        self.combine()

    def combine(self) -> None:
        self.densities.combine(self.species.uptake_weights, self.density)
        if self.species.produces:
            self.densities.combine(self.species.production, self.production)

    def sample_at_cells(self, population, out: torch.Tensor | None = None) -> None:
        """Trilinear interpolation into ``out`` (default: ``population.local_field(name)``)."""
        if population.count == 0:
            return
        target = out if out is not None else population.local_field(self.name)
        with profiling.stage("sample"):
            _lib.call("wbc_sample", ctypes.byref(self.geometry.native()), _lib.ptr(self.field.values),
                      population.count, _lib.ptr(population.position), _lib.ptr(target), _lib.stream(self.device))

    # ---- solvers --------------------------------------------------------------------------
    def solve_steady_state(self, source: SpeciesField | None = None, defer: bool = False):
        """The steady solve; with ``defer`` a PendingSolve whose ``result()`` gives the report
        (and records it as ``last_report``)."""
        return solve_steady_state(
            self.field, self.density, self.species.kinetics, self.settings, self._residual,
            production=self.production if self.species.produces else None,
            source=source.field.values if source is not None else None,
            source_k=source.species.michaelis_k if source is not None else 1.0,
            defer=defer, on_result=self._record_report,
        )

    def _record_report(self, report: SolveReport) -> None:
        self.last_report = report

    def explicit_step(self, dt: float, source: SpeciesField | None = None) -> None:
        explicit_step(
            self.field, self.density, self.species.kinetics, dt, self._scratch,
            production=self.production if self.species.produces else None,
            source=source.field.values if source is not None else None,
            source_k=source.species.michaelis_k if source is not None else 1.0,
        )

    def update(self, population, source: SpeciesField | None = None, out: torch.Tensor | None = None,
               defer: bool = False):
        """Deposit (if owner), combine, solve to steady state, sample: the per-cell-step update
        (with ``defer``, the solve's report as a PendingSolve)."""
        self.deposit_uptake(population)
        report = self.solve_steady_state(source, defer=defer)
        self.sample_at_cells(population, out)
        return report

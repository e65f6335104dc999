"""Several diffusible species on one grid that share one deposit of the per-state cell densities
(reference: fields/metabolism.py:27-111, whose class names, constructor parameters and report
properties these keep).

The species are kept in solve order, oxygen first. Each species is coupled to the cells through
its own per-state uptake (and production) weights over the shared densities; a species whose
production is scaled by another species' concentration (lactate from glucose) must come after it,
and reads that species' freshly solved field. Oxygen samples into ``oxygen_local``, glucose into
``glucose_local`` and any other species into ``population.extra_local[name]``.
"""

from __future__ import annotations

from dataclasses import dataclass

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.fields.densities import CellDensities
from warpbiocell_gb300.fields.diffusion import SolveReport, SolverSettings
from warpbiocell_gb300.fields.oxygen import OxygenField, OxygenParams
from warpbiocell_gb300.fields.scalar_field import Boundary, GridGeometry
from warpbiocell_gb300.fields.species import SpeciesField, SpeciesParams


@dataclass(frozen=True)
class MetabolicReport:
    """The solve reports of one update, by species name; the aggregate properties summarise them
    (total sweeps, worst residual, all converged)."""

    reports: dict

    def _all(self) -> list[SolveReport]:
        return list(self.reports.values())

    @property
    def sweeps(self) -> int:
        return sum(report.sweeps for report in self._all())

    @property
    def residual(self) -> float:
        return max(report.residual for report in self._all())

    @property
    def converged(self) -> bool:
        return all(report.converged for report in self._all())


class MetabolicFields:
    def __init__(self, geometry: GridGeometry, oxygen_params: OxygenParams, species: list[SpeciesParams],
                 settings: SolverSettings = SolverSettings(),
                 boundary: tuple[Boundary, Boundary, Boundary] = (Boundary.DIRICHLET,) * 3, device=None,
                 fixed_outside=None, oxygen_state_factors: dict | None = None):
        self.device = _lib.resolve_device(device)
        self.densities = CellDensities(geometry, device=self.device)
        # what every further species is built with
        self._field_options = dict(settings=settings, boundary=boundary, device=self.device,
                                   fixed_outside=fixed_outside, densities=self.densities)
        self.oxygen = OxygenField(geometry, oxygen_params, settings, boundary=boundary, device=self.device,
                                  fixed_outside=fixed_outside, densities=self.densities,
                                  uptake_state_factors=oxygen_state_factors)
        self.species_fields: dict[str, SpeciesField] = {"oxygen": self.oxygen}
        self._sources: dict[str, SpeciesField | None] = {"oxygen": None}
        for params in species:
            self.add_species(params)
        self.last_report: MetabolicReport | None = None

    def add_species(self, params: SpeciesParams) -> SpeciesField:
        """Append a species to the solve order (its production source, if any, must already be there)."""
        if params.name in self.species_fields:
            raise ValueError(f"duplicate species {params.name!r}")
        source = params.production_source
        if source is not None and source not in self.species_fields:
            raise ValueError(f"species {params.name!r}: production source {source!r} must be an earlier species")
        added = SpeciesField(self.geometry, params, **self._field_options)
        self.species_fields[params.name] = added
        self._sources[params.name] = None if source is None else self.species_fields[source]
        return added

    @property
    def geometry(self) -> GridGeometry:
        return self.oxygen.geometry

    @property
    def names(self) -> list[str]:
        return list(self.species_fields)

    @property
    def field(self):
        return self.oxygen.field

    def numpy(self):
        return self.oxygen.numpy()

    def __getitem__(self, name: str) -> SpeciesField:
        return self.species_fields[name]

    def update(self, population, defer: bool = False):
        """One deposit for all species, then, in order, each species' coupling, steady solve and
        sampling at the cells (with ``defer``, a pending report whose ``result()`` gives the
        MetabolicReport)."""
        self.densities.deposit(population)
        pending = {}
        for name, species in self.species_fields.items():
            species.combine()
            pending[name] = species.solve_steady_state(self._sources[name], defer=True)
            species.sample_at_cells(population)
        report = _PendingMetabolic(self, pending)
        return report if defer else report.result()


class _PendingMetabolic:
    """The species' deferred solves of one update; ``result()`` reads them all."""

    def __init__(self, fields: MetabolicFields, pending: dict):
        self._fields = fields
        self._pending = pending
        self._report: MetabolicReport | None = None

    def result(self) -> MetabolicReport:
        if self._report is None:
            reports = {name: p.result() for name, p in self._pending.items()}
            self._fields.oxygen.last_report = reports["oxygen"]
            self._report = MetabolicReport(reports)
            self._fields.last_report = self._report
        return self._report

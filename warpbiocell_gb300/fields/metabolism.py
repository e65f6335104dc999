"""Several diffusible species on one grid, sharing the per-state cell densities
(reference: fields/metabolism.py:27-111).

Oxygen is always first (the lifecycle reads ``oxygen_local``); glucose, when present, is sampled
into ``glucose_local``; other species into ``population.extra_local[name]``. Species are solved
in list order and may take their production source from an earlier species (lactate from
glucose).
"""

from __future__ import annotations

from dataclasses import dataclass

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.fields.densities import CellDensities
from warpbiocell_gb300.fields.diffusion import SolverSettings
from warpbiocell_gb300.fields.oxygen import OxygenField, OxygenParams
from warpbiocell_gb300.fields.scalar_field import Boundary, GridGeometry
from warpbiocell_gb300.fields.species import SpeciesField, SpeciesParams


@dataclass(frozen=True)
class MetabolicReport:
    reports: dict

    @property
    def sweeps(self) -> int:
        return sum(r.sweeps for r in self.reports.values())

    @property
    def residual(self) -> float:
        return max(r.residual for r in self.reports.values())

    @property
    def converged(self) -> bool:
        return all(r.converged for r in self.reports.values())


class MetabolicFields:
    def __init__(self, geometry: GridGeometry, oxygen_params: OxygenParams, species: list[SpeciesParams],
                 settings: SolverSettings = SolverSettings(),
                 boundary: tuple[Boundary, Boundary, Boundary] = (Boundary.DIRICHLET,) * 3, device=None,
                 fixed_outside=None, oxygen_state_factors: dict | None = None):
        self.device = _lib.resolve_device(device)
        self.densities = CellDensities(geometry, device=self.device)
        self.oxygen = OxygenField(geometry, oxygen_params, settings, boundary=boundary, device=self.device,
                                  fixed_outside=fixed_outside, densities=self.densities,
                                  uptake_state_factors=oxygen_state_factors)
        self.species_fields: dict[str, SpeciesField] = {"oxygen": self.oxygen}
        self._settings, self._boundary, self._fixed_outside = settings, boundary, fixed_outside
        for params in species:
            self.add_species(params)
        self.last_report: MetabolicReport | None = None

    def add_species(self, params: SpeciesParams) -> SpeciesField:
        """Append a species after oxygen (and after any species it takes its production from)."""
        if params.name in self.species_fields:
            raise ValueError(f"duplicate species {params.name!r}")
        if params.production_source is not None and params.production_source not in self.species_fields:
            raise ValueError(f"species {params.name!r}: production source {params.production_source!r} must be an earlier species")
        fld = SpeciesField(self.geometry, params, self._settings, boundary=self._boundary, device=self.device,
                           fixed_outside=self._fixed_outside, densities=self.densities)
        self.species_fields[params.name] = fld
        return fld

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

    def update(self, population) -> MetabolicReport:
        """Deposit the per-state densities once, then combine, solve and sample every species in order."""
        self.densities.deposit(population)
        reports = {}
        for name, species in self.species_fields.items():
            species.combine()
            source = self.species_fields[species.species.production_source] if species.species.production_source else None
            reports[name] = species.solve_steady_state(source)
            species.sample_at_cells(population)
        self.last_report = MetabolicReport(reports)
        self.oxygen.last_report = reports["oxygen"]
        return self.last_report

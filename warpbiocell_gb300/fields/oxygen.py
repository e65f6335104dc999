"""Oxygen field: parameters and the cell <-> field coupling (reference: fields/oxygen.py:20-103).

Oxygen partial pressure in mmHg (7.13 mmHg per % O2 at 37 C). Oxygen is a SpeciesField with
uniform uptake over the living states (optionally scaled per state with
``uptake_state_factors``) that samples into ``population.oxygen_local``.
"""

from __future__ import annotations

from dataclasses import dataclass

from warpbiocell_gb300.cells.model import CellState
from warpbiocell_gb300.fields.densities import CellDensities
from warpbiocell_gb300.fields.diffusion import SolverSettings, UptakeKinetics
from warpbiocell_gb300.fields.scalar_field import Boundary, GridGeometry
from warpbiocell_gb300.fields.species import SpeciesField, SpeciesParams, by_state

MMHG_PER_PERCENT_O2 = 7.13


@dataclass(frozen=True)
class OxygenParams:
    diffusion_coefficient: float = 7.2e6  # um^2/h
    uptake_max: float = 1.4e8  # mmHg um^3/h per living cell
    michaelis_k: float = 3.4  # mmHg
    boundary_value: float = 38.0  # mmHg

    def __post_init__(self):
        if self.boundary_value < 0.0:
            raise ValueError("boundary_value must be non-negative")
        self.kinetics  # validates the rest

    @property
    def kinetics(self) -> UptakeKinetics:
        return UptakeKinetics(self.diffusion_coefficient, self.uptake_max, self.michaelis_k)


class OxygenField(SpeciesField):
    def __init__(self, geometry: GridGeometry, params: OxygenParams, settings: SolverSettings = SolverSettings(),
                 boundary: tuple[Boundary, Boundary, Boundary] = (Boundary.DIRICHLET,) * 3, device=None,
                 fixed_outside=None, densities: CellDensities | None = None, uptake_state_factors: dict | None = None):
        self.oxygen_params = params
        super().__init__(geometry, species_params(params, uptake_state_factors), settings, boundary=boundary,
                         device=device, fixed_outside=fixed_outside, densities=densities)

    @property
    def params(self) -> OxygenParams:  # type: ignore[override]
        return self.oxygen_params

    def sample_at_cells(self, population, out=None) -> None:
        super().sample_at_cells(population, out if out is not None else population.oxygen_local)


def species_params(params: OxygenParams, uptake_state_factors: dict | None = None) -> SpeciesParams:
    factors = by_state(uptake_state_factors, default=1.0) if uptake_state_factors else (1.0, 1.0, 1.0, 0.0)
    uptake = tuple(params.uptake_max * f if k != int(CellState.DEAD) else 0.0 for k, f in enumerate(factors))
    return SpeciesParams(name="oxygen", unit="mmHg", diffusion=params.diffusion_coefficient,
                         michaelis_k=params.michaelis_k, boundary_value=params.boundary_value, uptake_max=uptake)

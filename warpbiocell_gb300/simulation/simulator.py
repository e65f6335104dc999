"""One cell step = field update, gene network, lifecycle decisions, mechanical relaxation
(reference: simulation/simulator.py:32-81).

Operator splitting, in this order:
    oxygen.update        deposit cells on the grid, solve the quasi-steady field(s) from the
                         previous solution, sample them at the cells (one host sync per residual
                         check)                                                   [optional]
    network.step         clamp inputs, advance every cell's network, pack fates  [optional]
    lifecycle_step       states, deaths, divisions; daughters appended (one host sync)
    network.inherit      daughters copy the parent's network                     [optional]
    relax_contacts       mechanics substeps, each rebinning the cells; leaves neighbor_count
                         for the next lifecycle decision
"""

from __future__ import annotations

from dataclasses import dataclass

from warpbiocell_gb300.cells.lifecycle import LifecycleParams, lifecycle_step
from warpbiocell_gb300.cells.mechanics import ContactParams, relax_contacts


@dataclass(frozen=True)
class TimeStepping:
    """dt_cells [h] per lifecycle update; dt_mechanics [h] per contact substep."""

    dt_cells: float = 0.25
    dt_mechanics: float = 0.025

    def __post_init__(self):
        if self.dt_cells <= 0.0 or self.dt_mechanics <= 0.0:
            raise ValueError("time steps must be positive")
        if self.dt_mechanics > self.dt_cells:
            raise ValueError("dt_mechanics cannot exceed dt_cells")

    @property
    def mechanics_substeps(self) -> int:
        return max(1, int(round(self.dt_cells / self.dt_mechanics)))


@dataclass(frozen=True)
class StepReport:
    daughters: int
    field_sweeps: int = 0
    field_residual: float = 0.0
    field_converged: bool = True


def cell_step(population, grid, lifecycle: LifecycleParams, contact: ContactParams, stepping: TimeStepping,
              oxygen=None, region=None, network=None) -> StepReport:
    """Advance the population by ``stepping.dt_cells``."""
    # The field solves are launched without waiting for their reports: the stream runs on into
    # the network and the lifecycle, and the reports are read once the division count (the
    # step's one synchronisation) has been read.
    pending = oxygen.update(population, defer=True) if oxygen is not None else None
    if network is not None:
        network.step(population, stepping.dt_cells)
    count_before = population.count
    n_daughters = lifecycle_step(population, lifecycle, stepping.dt_cells)
    if network is not None and n_daughters:
        network.inherit(population, count_before)
    relax_contacts(population, grid, contact, stepping.dt_mechanics, stepping.mechanics_substeps, region)
    if pending is None:
        return StepReport(n_daughters)
    fld = pending.result()
    return StepReport(n_daughters, fld.sweeps, fld.residual, fld.converged)

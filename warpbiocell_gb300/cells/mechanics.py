"""Overdamped contact mechanics: parameters, stability rule and the substep driver
(reference: cells/mechanics.py:17-122).

One substep = ``wbc_grid_build`` (binning) + ``wbc_contact_substep``, which counts neighbours,
gathers the overlap repulsion ``rate * overlap / d * (x_i - x_j)`` and moves the cells by
``v dt`` in one kernel (velocities are computed from the bucket-ordered snapshot of the
positions, so the in-place update is race free).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

from warpbiocell_gb300 import _lib, profiling
from warpbiocell_gb300.spatial.neighbors import NeighborGrid

# Explicit Euler on one overlapping pair contracts the overlap by (1 - 2 rate dt) per substep;
# above rate dt = 0.5 the pair overshoots, so it is refused.
MAX_RATE_DT = 0.5


@dataclass(frozen=True)
class ContactParams:
    """Linear repulsion between overlapping spheres, overdamped: only ``rate = k / gamma`` [1/h]
    enters the dynamics; ``query_radius = 2 max_radius + margin`` is the neighbour radius."""

    stiffness: float
    damping: float
    max_radius: float
    margin: float = 0.0
    wall_rate: float = 10.0

    def __post_init__(self):
        if self.stiffness <= 0.0 or self.damping <= 0.0:
            raise ValueError("stiffness and damping must be positive")
        if self.max_radius <= 0.0:
            raise ValueError("max_radius must be positive")
        if self.margin < 0.0:
            raise ValueError("margin must be non-negative")
        if self.wall_rate < 0.0:
            raise ValueError("wall_rate must be non-negative")

    @property
    def rate(self) -> float:
        return self.stiffness / self.damping

    @property
    def query_radius(self) -> float:
        return 2.0 * self.max_radius + self.margin

    def check_substep(self, dt: float) -> None:
        if dt <= 0.0:
            raise ValueError("dt must be positive")
        if self.rate * dt > MAX_RATE_DT:
            raise ValueError(
                f"rate*dt = {self.rate * dt:.3g} exceeds {MAX_RATE_DT}: explicit contact relaxation "
                "would overshoot. Reduce dt_mechanics or stiffness/damping."
            )
        if self.wall_rate * dt > MAX_RATE_DT:
            raise ValueError(f"wall_rate*dt = {self.wall_rate * dt:.3g} exceeds {MAX_RATE_DT}: reduce dt_mechanics or wall_rate.")


def make_neighbor_grid(params: ContactParams, device, dim: int = 128) -> NeighborGrid:
    return NeighborGrid(cell_size=params.query_radius, dim=dim, device=device)


def contact_substep(population, grid: NeighborGrid, params: ContactParams, dt: float, region=None) -> None:
    """One explicit substep: rebuild the grid, gather contact velocities, move the cells."""
    n = population.count
    if n == 0:
        return
    grid.build(population)
    with profiling.stage("contact"):
        if region is None:
            _lib.call("wbc_contact_substep", ctypes.byref(grid.struct), n, float(params.query_radius),
                      float(params.rate), float(dt), _lib.ptr(population.position), _lib.ptr(population.velocity),
                      _lib.ptr(population.neighbor_count), _lib.stream(population.device))
        else:
            if region.device != population.device:
                raise RuntimeError("population and tissue region must live on the same device")
            native = region.native(params.wall_rate)
            _lib.call("wbc_contact_substep_region", ctypes.byref(grid.struct), n, float(params.query_radius),
                      float(params.rate), float(dt), ctypes.byref(native), _lib.ptr(population.position),
                      _lib.ptr(population.velocity), _lib.ptr(population.neighbor_count),
                      _lib.stream(population.device))


def relax_contacts(population, grid: NeighborGrid, params: ContactParams, dt: float, substeps: int, region=None) -> None:
    params.check_substep(dt)
    for _ in range(substeps):
        contact_substep(population, grid, params, dt, region)

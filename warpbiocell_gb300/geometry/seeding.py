"""Initial cells filling a tissue region (reference: geometry/seeding.py, whose function name,
parameters, exception and point pattern these keep, so a seeded configuration places the same
cells).

The cells start on a cubic lattice of pitch ``spacing_factor`` cell diameters that begins half a
pitch inside the grid's lower corner, each lattice point moved by an independent uniform jitter
of up to ``jitter`` radii per axis (one ``numpy.random.default_rng(seed)`` draw for all of them);
a point is kept when a whole cell (plus ``margin``) fits inside the region, and inside the
optional sub-volume ``within``.
"""

from __future__ import annotations

import numpy as np

from warpbiocell_gb300.geometry.region import TissueRegion


class CellBudgetError(ValueError):
    """The region holds more cells than the run is allowed to allocate."""


def _lattice(low, high, pitch: float) -> np.ndarray:
    """(n, 3) lattice points from low + pitch / 2 up to high, x slowest, z fastest."""
    axes = [np.arange(a + 0.5 * pitch, b, pitch) for a, b in zip(low, high)]
    return np.column_stack([g.reshape(-1) for g in np.meshgrid(*axes, indexing="ij")])


def fill_region(region: TissueRegion, radius: float, spacing_factor: float = 1.0, jitter: float = 0.1, seed: int = 0,
                margin: float = 0.0, max_cells: int | None = None, within=None) -> np.ndarray:
    """Positions [um] (float32, (n, 3)) of the cells seeded inside ``region``; more than
    ``max_cells`` of them raise :class:`CellBudgetError`."""
    if not radius > 0.0:
        raise ValueError("radius must be positive")
    pitch = spacing_factor * 2.0 * radius
    points = _lattice(region.geometry.origin, region.geometry.upper, pitch)
    wobble = jitter * radius
    points = points + np.random.default_rng(seed).uniform(-wobble, wobble, size=points.shape)
    clearance = radius + margin
    inside = region.contains(points, margin=clearance)
    if within is not None:
        inside &= within.sdf(points[:, 0], points[:, 1], points[:, 2]) < -clearance
    cells = points[inside]
    if max_cells is not None and len(cells) > max_cells:
        raise CellBudgetError(f"the region holds {len(cells)} cells at this spacing, more than the budget of "
                              f"{max_cells}: seed a smaller sub-volume (within=...), allow more cells, or space "
                              "them further apart")
    return cells.astype(np.float32)

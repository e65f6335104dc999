"""Seed cells inside a tissue region (reference: geometry/seeding.py)."""

from __future__ import annotations

import numpy as np

from warpbiocell_gb300.geometry.region import TissueRegion


class CellBudgetError(ValueError):
    """The region holds more cells than the run is allowed to allocate."""


def fill_region(region: TissueRegion, radius: float, spacing_factor: float = 1.0, jitter: float = 0.1, seed: int = 0,
                margin: float = 0.0, max_cells: int | None = None, within=None) -> np.ndarray:
    """Positions [um] of cells on a jittered cubic lattice inside the region.

    The lattice has spacing ``spacing_factor * 2 * radius`` from half a spacing inside the grid's
    lower corner; each point moves by a uniform jitter of up to ``jitter * radius`` per axis
    (``numpy.random.default_rng(seed)``) and is kept when it lies at least ``radius + margin``
    inside the surface and, with ``within`` (a shape), inside that sub-volume too. More than
    ``max_cells`` points raise :class:`CellBudgetError`.
    """
    if radius <= 0.0:
        raise ValueError("radius must be positive")
    rng = np.random.default_rng(seed)
    spacing = spacing_factor * 2.0 * radius
    lo, hi = np.asarray(region.geometry.origin), np.asarray(region.geometry.upper)
    axes = [np.arange(lo[a] + 0.5 * spacing, hi[a], spacing) for a in range(3)]
    gx, gy, gz = np.meshgrid(*axes, indexing="ij")
    points = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)
    points += rng.uniform(-jitter * radius, jitter * radius, size=points.shape)
    keep = region.contains(points, margin=radius + margin)
    if within is not None:
        keep &= within.sdf(points[:, 0], points[:, 1], points[:, 2]) < -(radius + margin)
    points = points[keep]
    if max_cells is not None and points.shape[0] > max_cells:
        raise CellBudgetError(
            f"the region holds {points.shape[0]} cells at this packing, above the budget of {max_cells}; "
            "seed a sub-volume (within=...), raise the cell budget or coarsen the representation")
    return points.astype(np.float32)

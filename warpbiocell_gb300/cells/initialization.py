"""Initial cell configurations (host numpy; reference: cells/initialization.py:8-38)."""

from __future__ import annotations

import numpy as np


def spherical_cluster(
    n_cells: int,
    radius: float,
    spacing_factor: float = 0.9,
    jitter: float = 0.1,
    seed: int = 0,
) -> np.ndarray:
    """``(n_cells, 3)`` float32 positions [um]: the ``n_cells`` points of a cubic lattice of spacing
    ``spacing_factor * 2 * radius`` nearest the origin (stable order by squared distance), each
    displaced by uniform jitter in ``[-jitter * radius, jitter * radius]`` drawn from
    ``numpy.random.default_rng(seed)``. The lattice keeps centres distinct, which the contact
    law needs (coincident centres have no separation direction)."""
    if n_cells <= 0:
        raise ValueError("n_cells must be positive")
    rng = np.random.default_rng(seed)
    step = spacing_factor * 2.0 * radius
    # Half-width (in lattice steps) of a cube whose inscribed ball holds n_cells points.
    side = (n_cells / (np.pi / 6.0)) ** (1.0 / 3.0)
    half = int(np.ceil(side / 2.0)) + 1
    ticks = np.arange(-half, half + 1, dtype=np.float64) * step
    grid = np.stack(np.meshgrid(ticks, ticks, ticks, indexing="ij"), axis=-1).reshape(-1, 3)
    nearest = np.argsort(np.einsum("ij,ij->i", grid, grid), kind="stable")[:n_cells]
    points = grid[nearest]
    points = points + rng.uniform(-jitter * radius, jitter * radius, size=points.shape)
    return points.astype(np.float32)


def uniform_ball(n_cells: int, ball_radius: float, seed: int = 0) -> np.ndarray:
    """``(n_cells, 3)`` float32 positions uniform in a ball: r = R u^(1/3) along an isotropic
    direction (normalised Gaussian triple), from ``numpy.random.default_rng(seed)``. The
    synthetic spheroids of the benchmark workloads use it."""
    if n_cells <= 0:
        raise ValueError("n_cells must be positive")
    rng = np.random.default_rng(seed)
    direction = rng.normal(size=(n_cells, 3))
    direction /= np.linalg.norm(direction, axis=1, keepdims=True)
    r = ball_radius * rng.random(n_cells) ** (1.0 / 3.0)
    return (direction * r[:, None]).astype(np.float32)


def clipped_normal_radii(n_cells: int, mean: float = 8.0, sd: float = 0.8, lo: float = 6.0, hi: float = 10.0,
                         seed: int = 0) -> np.ndarray:
    """Radii N(mean, sd) clipped to [lo, hi] [um], float32."""
    rng = np.random.default_rng(seed)
    return np.clip(rng.normal(mean, sd, size=n_cells), lo, hi).astype(np.float32)

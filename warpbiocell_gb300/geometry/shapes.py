"""Analytical tissue shapes as signed distances (negative inside), in um, for tissue regions
(reference: geometry/shapes.py, whose class names, fields and defaults these keep).

Every shape answers three questions: the signed distance at points, the axis-aligned box that
contains it, and its volume. The sphere's distance is exact. For the ellipsoid with semi-axes
a the distance is the first-order estimate of its implicit function |(x - c) / a| - 1,
g (g - 1) / |(x - c) / a^2| with g = |(x - c) / a| (exact on the axes, within a few percent
elsewhere for moderate aspect ratios; at the centre, where the gradient vanishes, it is minus the
smallest semi-axis). A union is the pointwise minimum of its members' distances.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from warpbiocell_gb300.fields.scalar_field import GridGeometry


def _norm(u, v, w):
    return np.sqrt(u**2 + v**2 + w**2)


def _relative(center, scale, x, y, z):
    """The coordinates relative to ``center``, each divided by its ``scale``."""
    return [(q - c) / s for q, c, s in zip((x, y, z), center, scale)]


class _Shape:
    """Shared helpers of the shapes (each defines ``sdf``, ``bounds`` and ``volume``)."""

    def sdf_points(self, points: np.ndarray) -> np.ndarray:
        """Signed distance at an (..., 3) array of points."""
        points = np.asarray(points, dtype=float)
        return self.sdf(points[..., 0], points[..., 1], points[..., 2])

    def contains(self, points: np.ndarray) -> np.ndarray:
        return self.sdf_points(points) < 0.0


@dataclass(frozen=True)
class Sphere(_Shape):
    center: tuple[float, float, float] = (0.0, 0.0, 0.0)
    radius: float = 200.0

    def __post_init__(self):
        if not self.radius > 0.0:
            raise ValueError("radius must be positive")

    def sdf(self, x, y, z) -> np.ndarray:
        return _norm(*_relative(self.center, (1.0, 1.0, 1.0), x, y, z)) - self.radius

    @property
    def bounds(self) -> tuple[np.ndarray, np.ndarray]:
        half = np.full(3, float(self.radius))
        return np.asarray(self.center, dtype=float) - half, np.asarray(self.center, dtype=float) + half

    @property
    def volume(self) -> float:
        return 4.0 / 3.0 * np.pi * self.radius**3


@dataclass(frozen=True)
class Ellipsoid(_Shape):
    center: tuple[float, float, float] = (0.0, 0.0, 0.0)
    radii: tuple[float, float, float] = (300.0, 200.0, 150.0)  # semi-axes

    def __post_init__(self):
        if not min(self.radii) > 0.0:
            raise ValueError("semi-axes must be positive")

    def sdf(self, x, y, z) -> np.ndarray:
        u = _relative(self.center, self.radii, x, y, z)
        g = _norm(*u)
        grad = _norm(*(ui / a for ui, a in zip(u, self.radii)))
        inside_centre = -min(self.radii)
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(grad > 0.0, g * (g - 1.0) / grad, inside_centre)

    @property
    def bounds(self) -> tuple[np.ndarray, np.ndarray]:
        half = np.asarray(self.radii, dtype=float)
        return np.asarray(self.center, dtype=float) - half, np.asarray(self.center, dtype=float) + half

    @property
    def volume(self) -> float:
        a, b, c = self.radii
        return 4.0 / 3.0 * np.pi * float(a * b * c)


@dataclass(frozen=True)
class Union(_Shape):
    shapes: tuple = field(default_factory=tuple)

    def __post_init__(self):
        if len(self.shapes) == 0:
            raise ValueError("a union needs at least one shape")

    def sdf(self, x, y, z) -> np.ndarray:
        distance = self.shapes[0].sdf(x, y, z)
        for member in self.shapes[1:]:
            distance = np.minimum(distance, member.sdf(x, y, z))
        return distance

    @property
    def bounds(self) -> tuple[np.ndarray, np.ndarray]:
        boxes = [member.bounds for member in self.shapes]
        return np.min([lo for lo, _ in boxes], axis=0), np.max([hi for _, hi in boxes], axis=0)

    @property
    def volume(self) -> float:
        """Not known analytically (the members may overlap): NaN; measure it on a grid."""
        return float("nan")


def evaluate_on_grid(shape, geometry: GridGeometry) -> np.ndarray:
    """The signed distance at every node of ``geometry``, float32 (nx, ny, nz)."""
    xs, ys, zs = geometry.node_coordinates()
    return shape.sdf(xs[:, None, None], ys[None, :, None], zs[None, None, :]).astype(np.float32)

"""Regular 3-D scalar grid with per-axis boundary conditions (reference: fields/scalar_field.py:24-150).

Node ``(i, j, k)`` sits at ``origin + dx * (i, j, k)``; values are a float32 torch tensor of
shape ``(nx, ny, nz)`` (k fastest). A DIRICHLET axis holds ``boundary_value`` on its two face
planes, which solvers never write; a NEUMANN axis mirrors. Further nodes can be pinned with
``set_fixed`` (int32 mask, 1 = pinned).
"""

from __future__ import annotations

from dataclasses import dataclass
from enum import IntEnum

import numpy as np
import torch

from warpbiocell_gb300 import _lib


class Boundary(IntEnum):
    DIRICHLET = 0
    NEUMANN = 1


@dataclass(frozen=True)
class GridGeometry:
    origin: tuple[float, float, float]
    dx: float
    shape: tuple[int, int, int]

    def __post_init__(self):
        if self.dx <= 0.0:
            raise ValueError("dx must be positive")
        if len(self.shape) != 3 or min(self.shape) < 3:
            raise ValueError("shape needs at least 3 nodes per axis")

    @classmethod
    def centered_cube(cls, side: float, dx: float) -> GridGeometry:
        """Cube of edge ``side`` [um] centred on the origin; ``side`` is rounded up to whole voxels."""
        n = int(np.ceil(side / dx)) + 1
        half = 0.5 * (n - 1) * dx
        return cls(origin=(-half, -half, -half), dx=dx, shape=(n, n, n))

    @property
    def node_count(self) -> int:
        return int(np.prod(self.shape))

    @property
    def voxel_volume(self) -> float:
        return self.dx**3

    @property
    def upper(self) -> tuple[float, float, float]:
        return tuple(self.origin[a] + self.dx * (self.shape[a] - 1) for a in range(3))

    def node_coordinates(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        return tuple(self.origin[a] + self.dx * np.arange(self.shape[a]) for a in range(3))

    def contains(self, positions: np.ndarray) -> np.ndarray:
        """Boolean mask of positions inside the trilinear support of the grid."""
        p = np.asarray(positions)
        lo = np.asarray(self.origin)
        hi = np.asarray(self.upper)
        return np.all((p >= lo) & (p <= hi), axis=1)

    def native(self) -> _lib.GridGeometryC:
        """Kernel view: float32 origin and 1/dx (rounded from double, as the reference's launch does)."""
        nx, ny, nz = self.shape
        return _lib.GridGeometryC(nx=nx, ny=ny, nz=nz, origin_x=self.origin[0], origin_y=self.origin[1],
                                  origin_z=self.origin[2], inv_dx=1.0 / self.dx)


@dataclass
class ScalarField:
    geometry: GridGeometry
    boundary: tuple[Boundary, Boundary, Boundary]
    boundary_value: float
    device: torch.device
    values: torch.Tensor  # (nx, ny, nz) float32
    fixed: torch.Tensor  # (nx, ny, nz) int32, 1 where pinned to boundary_value

    @classmethod
    def create(cls, geometry: GridGeometry, boundary_value: float,
               boundary: tuple[Boundary, Boundary, Boundary] = (Boundary.DIRICHLET,) * 3,
               initial_value: float | None = None, device=None) -> ScalarField:
        dev = _lib.resolve_device(device)
        fill = boundary_value if initial_value is None else initial_value
        values = torch.full(geometry.shape, float(fill), dtype=torch.float32, device=dev)
        fixed = torch.zeros(geometry.shape, dtype=torch.int32, device=dev)
        field = cls(geometry=geometry, boundary=tuple(Boundary(b) for b in boundary),
                    boundary_value=float(boundary_value), device=dev, values=values, fixed=fixed)
        field.apply_dirichlet()
        return field

    def set_fixed(self, mask: np.ndarray | None) -> None:
        """Pin the nodes where ``mask`` is true to ``boundary_value`` (``None`` clears the mask)."""
        if mask is None:
            self.fixed.zero_()
            object.__setattr__(self, "_any_fixed", False)
            return
        mask = np.asarray(mask, dtype=bool)
        if mask.shape != tuple(self.geometry.shape):
            raise ValueError(f"mask shape {mask.shape} does not match the grid {self.geometry.shape}")
        self.fixed.copy_(torch.from_numpy(mask.astype(np.int32)))
        object.__setattr__(self, "_any_fixed", bool(mask.any()))
        self.apply_dirichlet()

    @property
    def any_fixed(self) -> bool:
        """True once a node has been pinned with ``set_fixed`` (solvers then read the mask)."""
        return getattr(self, "_any_fixed", False)

    def fixed_or_none(self) -> torch.Tensor | None:
        """The pin mask for the kernels, or None when nothing is pinned (the mask is not read)."""
        return self.fixed if self.any_fixed else None

    def fixed_mask(self) -> np.ndarray:
        return self.fixed.cpu().numpy().astype(bool)

    def fixed_zero_like(self) -> torch.Tensor:
        zero = getattr(self, "_zero", None)
        if zero is None:
            zero = torch.zeros(self.geometry.shape, dtype=torch.float32, device=self.device)
            object.__setattr__(self, "_zero", zero)
        return zero

    @property
    def boundary_flags(self) -> tuple[int, int, int]:
        return tuple(int(b) for b in self.boundary)

    def numpy(self) -> np.ndarray:
        return self.values.cpu().numpy().copy()

    def assign(self, array: np.ndarray) -> None:
        """Overwrite the values (Dirichlet faces are re-imposed afterwards)."""
        array = np.ascontiguousarray(array, dtype=np.float32)
        if array.shape != tuple(self.geometry.shape):
            raise ValueError(f"expected shape {self.geometry.shape}, got {array.shape}")
        self.values.copy_(torch.from_numpy(array))
        self.apply_dirichlet()

    def apply_dirichlet(self) -> None:
        """Re-impose ``boundary_value`` on every Dirichlet face and pinned node (not per step)."""
        pinned = ~self.interior_mask_tensor()
        self.values.masked_fill_(pinned, self.boundary_value)

    def interior_mask_tensor(self) -> torch.Tensor:
        mask = torch.ones(self.geometry.shape, dtype=torch.bool, device=self.device)
        for axis, b in enumerate(self.boundary):
            if b == Boundary.DIRICHLET:
                mask.select(axis, 0).fill_(False)
                mask.select(axis, self.geometry.shape[axis] - 1).fill_(False)
        return mask & (self.fixed == 0)

    def interior_mask(self) -> np.ndarray:
        """Mask of nodes that solvers update (everything except Dirichlet faces and pinned nodes)."""
        return self.interior_mask_tensor().cpu().numpy()

"""A tissue region: a signed-distance field on a regular grid, negative inside (reference:
geometry/region.py). It confines cells (``contact_substep(..., region=...)``, the wall push of
``wbc_contact_substep_region``), pins the field outside the tissue (``fixed_outside``) and
seeds cells (``seeding.fill_region``)."""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.fields.scalar_field import GridGeometry
from warpbiocell_gb300.geometry.shapes import evaluate_on_grid


def node_gradient(values: np.ndarray, dx: float) -> np.ndarray:
    """Central differences inside, one-sided at the faces; shape (nx, ny, nz, 3), float32."""
    grads = np.gradient(values.astype(np.float64), dx, edge_order=1)
    return np.stack(grads, axis=-1).astype(np.float32)


class TissueRegion:
    def __init__(self, geometry: GridGeometry, sdf: np.ndarray, device=None, name: str = "region"):
        sdf = np.ascontiguousarray(sdf, dtype=np.float32)
        if sdf.shape != tuple(geometry.shape):
            raise ValueError(f"sdf shape {sdf.shape} does not match the grid {geometry.shape}")
        self.geometry = geometry
        self.name = name
        self._requested_device = device
        self._sdf_np = sdf
        self._device_arrays = None  # (sdf, gradient) on the device, made on first use

    @property
    def sdf(self) -> torch.Tensor:
        return self._arrays()[0]

    @property
    def gradient(self) -> torch.Tensor:
        """Node gradient of the distance, float32 (nx, ny, nz, 3)."""
        return self._arrays()[1]

    @property
    def device(self) -> torch.device:
        """Resolved on first device use, so the host-side queries need no GPU."""
        return _lib.resolve_device(self._requested_device)

    def _arrays(self):
        if self._device_arrays is None:
            self._device_arrays = (torch.from_numpy(self._sdf_np).to(self.device),
                                   torch.from_numpy(node_gradient(self._sdf_np, self.geometry.dx)).to(self.device))
        return self._device_arrays

    @classmethod
    def from_shape(cls, shape, geometry: GridGeometry, device=None) -> TissueRegion:
        return cls(geometry, evaluate_on_grid(shape, geometry), device=device, name=type(shape).__name__.lower())

    def native(self, wall_rate: float) -> _lib.TissueRegionC:
        return _lib.TissueRegionC(self.geometry.native(), _lib.ptr(self.sdf), _lib.ptr(self.gradient),
                                  float(wall_rate))

    # ---- host-side queries ---------------------------------------------------------------------
    def sdf_numpy(self) -> np.ndarray:
        return self._sdf_np.copy()

    def inside_mask(self) -> np.ndarray:
        """Nodes strictly inside the tissue."""
        return self._sdf_np < 0.0

    def volume(self) -> float:
        """Tissue volume [um^3] counted in whole voxels."""
        return float(self.inside_mask().sum()) * self.geometry.voxel_volume

    def sample(self, positions: np.ndarray) -> np.ndarray:
        """Trilinear signed distance at points [um] (host, float64); points outside the grid are clamped."""
        geom = self.geometry
        u = (np.asarray(positions, dtype=np.float64) - np.asarray(geom.origin)) / geom.dx
        u = np.clip(u, 0.0, np.array(geom.shape) - 1.0)
        base = np.minimum(np.floor(u).astype(int), np.array(geom.shape) - 2)
        f = u - base
        v = self._sdf_np.astype(np.float64)
        i, j, k = base[:, 0], base[:, 1], base[:, 2]
        fx, fy, fz = f[:, 0], f[:, 1], f[:, 2]
        c00 = v[i, j, k] * (1 - fx) + v[i + 1, j, k] * fx
        c10 = v[i, j + 1, k] * (1 - fx) + v[i + 1, j + 1, k] * fx
        c01 = v[i, j, k + 1] * (1 - fx) + v[i + 1, j, k + 1] * fx
        c11 = v[i, j + 1, k + 1] * (1 - fx) + v[i + 1, j + 1, k + 1] * fx
        return (c00 * (1 - fy) + c10 * fy) * (1 - fz) + (c01 * (1 - fy) + c11 * fy) * fz

    def contains(self, positions: np.ndarray, margin: float = 0.0) -> np.ndarray:
        """True where a point lies at least ``margin`` [um] inside the surface."""
        return self.sample(positions) < -margin

    # ---- device-side queries -------------------------------------------------------------------
    def sample_at(self, position: torch.Tensor, count: int, out: torch.Tensor) -> None:
        """float32 signed distance at the first ``count`` positions (device)."""
        if count > 0:
            native = self.native(0.0)
            _lib.call("wbc_sample_sdf", ctypes.byref(native), int(count), _lib.ptr(position), _lib.ptr(out),
                      _lib.stream(self.device))

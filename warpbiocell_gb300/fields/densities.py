"""Per-state cell number densities on the grid (reference: fields/densities.py:13-56).

``deposit`` adds every cell's trilinear weights as int64 fixed point (2^24 per cell) into
``accumulator[state]`` with ``wbc_deposit`` — integer atomics, so the result is bit-exact and
independent of thread order — then converts to ``density[state]`` [cells/um^3]. The conversion
also clears the accumulator for the next deposit, so no separate memset pass is needed.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from warpbiocell_gb300 import _lib, profiling
from warpbiocell_gb300.cells.model import NUM_STATES
from warpbiocell_gb300.fields.scalar_field import GridGeometry


class CellDensities:
    """``density[k]`` [cells/um^3] of cells in state ``k``."""

    def __init__(self, geometry: GridGeometry, device=None):
        if NUM_STATES != 4:
            raise RuntimeError("combine_densities assumes four cell states")
        self.geometry = geometry
        self.device = _lib.resolve_device(device)
        shape = (NUM_STATES, *geometry.shape)
        self._accumulator = torch.zeros(shape, dtype=torch.int64, device=self.device)
        self.density = torch.zeros(shape, dtype=torch.float32, device=self.device)
        self._native = geometry.native()

    @property
    def accumulator(self) -> torch.Tensor:
        """The int64 fixed-point accumulator (zero between deposits)."""
        return self._accumulator

    def deposit_fixed_point(self, population) -> None:
        """Add the cells' weights to the (cleared) accumulator without converting."""
        if population.device != self.device:
            raise RuntimeError("population and CellDensities must live on the same device")
        if population.count > 0:
            with profiling.stage("deposit"):
                _lib.call("wbc_deposit", ctypes.byref(self._native), population.count, _lib.ptr(population.position),
                          _lib.ptr(population.cell_state), _lib.ptr(self._accumulator), _lib.stream(self.device))

    def convert(self, weights=None, combined: torch.Tensor | None = None) -> None:
        """density = acc / 2^24 / dx^3 (and optionally combined = sum_k w_k density_k); clears acc."""
        w = None
        if weights is not None:
            w = (ctypes.c_float * 4)(*[float(x) for x in weights])
        with profiling.stage("convert"):
            _lib.call("wbc_density_convert", self.geometry.node_count, _lib.ptr(self._accumulator),
                      1.0 / self.geometry.voxel_volume, _lib.ptr(self.density), w, _lib.ptr(combined), 1,
                      _lib.stream(self.device))

    def deposit(self, population) -> None:
        self.deposit_fixed_point(population)
        self.convert()

    def combine(self, weights, out: torch.Tensor) -> None:
        """``out = sum_k weights[k] * density[k]`` (weights indexed by CellState)."""
        weights = [float(w) for w in weights]
        if len(weights) != NUM_STATES:
            raise ValueError(f"need {NUM_STATES} weights, got {len(weights)}")
        w = (ctypes.c_float * 4)(*weights)
        _lib.call("wbc_density_combine", self.geometry.node_count, w, _lib.ptr(self.density), _lib.ptr(out),
                  _lib.stream(self.device))

    def numpy(self) -> np.ndarray:
        return self.density.cpu().numpy().copy()

    def total_numpy(self) -> np.ndarray:
        return self.density.cpu().numpy().sum(axis=0)

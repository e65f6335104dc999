"""Per-state cell number densities on the grid (reference: fields/densities.py:13-56).

``deposit_fixed_point`` adds every cell's trilinear weights as fixed point (2^24 per cell) into a
32-bit accumulator with exact wrap counts (``wbc_deposit32``): integer atomics, so the sums are
bit-exact and independent of thread order, the same as the reference's int64 accumulator in half
the bytes. The cells are visited in the hash grid's order when the population
was binned at its current size, so that the atomics of a warp's cells hit nearby lines. The call
clears the accumulator first; it then keeps the deposit until the next one.

``convert`` produces the per-state densities [cells/um^3] (and optionally a weighted combination
in the same pass); ``convert_combined`` produces only the combination, for the plain oxygen step,
and leaves the per-state densities to be produced from the same deposit when ``density`` is read.
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
        nodes = geometry.node_count
        nbytes = int(_lib.load().wbc_deposit32_bytes(nodes))
        raw = torch.zeros(nbytes + 16, dtype=torch.uint8, device=self.device)
        off = (-raw.data_ptr()) % 16
        self._acc = raw[off:off + nbytes]
        self._planes = torch.zeros((NUM_STATES, *geometry.shape), dtype=torch.float32, device=self.device)
        self._planes_current = True  # the planes hold the densities of the latest deposit
        self._native = geometry.native()

    # ---- views ---------------------------------------------------------------------------------
    @property
    def density(self) -> torch.Tensor:
        """Per-state densities of the latest deposit, (4, nx, ny, nz) float32."""
        if not self._planes_current:
            self._convert(self._planes, None, None)
            self._planes_current = True
        return self._planes

    @property
    def accumulator(self) -> torch.Tensor:
        """The latest deposit's fixed-point sums as int64 (4, nx, ny, nz) (a copy, for inspection)."""
        words = 4 * self.geometry.node_count
        u32 = self._acc[: 8 * words].view(torch.int32)
        value = u32[:words].to(torch.int64) & 0xFFFFFFFF
        if int(self._acc[8 * words: 8 * words + 4].view(torch.int32).item()):
            # low words are added to in pairs (2m, 2m+1) by 64-bit atomics: a wrap of word 2m
            # carries into word 2m+1 and is counted in count[2m]; a wrap out of the pair in count[2m+1]
            count = u32[words:].to(torch.int64) & 0xFFFFFFFF
            value = value + (count << 32)
            value[1::2] -= count[0::2]
        return value.reshape(NUM_STATES, *self.geometry.shape)

    # ---- deposit and conversion ------------------------------------------------------------------
    def deposit_fixed_point(self, population) -> None:
        """Replace the accumulator's contents with the cells' weights (without converting)."""
        if population.device != self.device:
            raise RuntimeError("population and CellDensities must live on the same device")
        order = population.spatial_order()
        with profiling.stage("deposit", launches=2):
            _lib.call("wbc_deposit32", ctypes.byref(self._native), population.count, _lib.ptr(population.position),
                      _lib.ptr(population.cell_state), _lib.ptr(order), _lib.ptr(self._acc), self._acc.numel(),
                      _lib.stream(self.device))
        self._planes_current = False

    def _convert(self, density, weights, combined) -> None:
        w = None
        if weights is not None:
            w = (ctypes.c_float * 4)(*[float(x) for x in weights])
        with profiling.stage("convert"):
            _lib.call("wbc_convert32", self.geometry.node_count, _lib.ptr(self._acc), 1.0 / self.geometry.voxel_volume,
                      _lib.ptr(density), w, _lib.ptr(combined), _lib.stream(self.device))

    def convert(self, weights=None, combined: torch.Tensor | None = None) -> None:
        """density = acc / 2^24 / dx^3 (and optionally combined = sum_k w_k density_k)."""
        self._convert(self._planes, weights, combined)
        self._planes_current = True

    def convert_combined(self, weights, combined: torch.Tensor) -> None:
        """Only ``combined = sum_k weights[k] density_k``; the per-state densities are produced from
        the same deposit if and when ``density`` is read."""
        self._convert(None, weights, combined)

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

    def accumulator_for_writing(self) -> torch.Tensor:
        """The 32-bit accumulator, for a caller that deposits into it itself (the batched step); the
        per-state densities are then converted from it when ``density`` is read."""
        self._planes_current = False
        return self._acc

    def numpy(self) -> np.ndarray:
        return self.density.cpu().numpy().copy()

    def total_numpy(self) -> np.ndarray:
        return self.density.cpu().numpy().sum(axis=0)

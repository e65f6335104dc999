"""Neighbour search over the active cells of a population (reference: spatial/neighbors.py:16-37).

``NeighborGrid(cell_size, dim)`` hashes cells into ``dim**3`` buckets of edge ``cell_size``
(widened by 2^-10 against rounding) by a stable counting sort on the GPU (``wbc_grid_build``):
bucket counts, a prefix sum, a scatter and an in-bucket ordering by slot, plus a float4
(x, y, z, r) copy in bucket order that the contact kernel reads coalesced. ``dim`` sets the
bucket count, not the spatial extent: any position hashes somewhere, and the distance test in
the contact kernel removes the far cells that share a bucket. Bucket bookkeeping costs
``2 * 4 bytes * dim**3``; the per-cell buffers grow to the population's capacity on first use.
"""

from __future__ import annotations

import ctypes

import torch

from warpbiocell_gb300 import _lib, profiling


class NeighborGrid:
    def __init__(self, cell_size: float, dim: int = 128, device=None):
        """``cell_size`` [um] is the bucket edge and should equal the query radius used in kernels."""
        if cell_size <= 0.0:
            raise ValueError("cell_size must be positive")
        if dim < 3:
            raise ValueError("dim must be at least 3")
        self.cell_size = float(cell_size)
        self.dim = int(dim)
        self.device = _lib.resolve_device(device)
        buckets = self.dim**3
        self.bucket_count = torch.zeros(buckets, dtype=torch.int32, device=self.device)
        self.bucket_start = torch.zeros(buckets, dtype=torch.int32, device=self.device)
        nbytes = int(_lib.load().wbc_scan_workspace_bytes(buckets))
        self.scan_partials = torch.zeros((nbytes + 3) // 4, dtype=torch.int32, device=self.device)
        self._capacity = 0
        self._struct = _lib.NeighborGridC()
        self.reserve(1)

    @property
    def id(self) -> int:
        """Address of the native grid descriptor (the counterpart of the HashGrid handle)."""
        return ctypes.addressof(self._struct)

    @property
    def struct(self) -> _lib.NeighborGridC:
        return self._struct

    def reserve(self, num_points: int) -> None:
        """Size the per-cell buffers for ``num_points`` cells (grows only)."""
        if num_points <= self._capacity:
            return
        cap = int(num_points)
        dev = self.device
        self.cell_bucket = torch.empty(cap, dtype=torch.int32, device=dev)
        self.cell_rank = torch.empty(cap, dtype=torch.int32, device=dev)
        self.scatter = torch.empty(cap, dtype=torch.int32, device=dev)
        self.sorted_id = torch.empty(cap, dtype=torch.int32, device=dev)
        self.sorted_xyzr = torch.empty((cap, 4), dtype=torch.float32, device=dev)
        self._capacity = cap
        s = self._struct
        s.dim = self.dim
        s.cell_size = self.cell_size
        s.bucket_count = _lib.ptr(self.bucket_count)
        s.bucket_start = _lib.ptr(self.bucket_start)
        s.cell_bucket = _lib.ptr(self.cell_bucket)
        s.cell_rank = _lib.ptr(self.cell_rank)
        s.scatter = _lib.ptr(self.scatter)
        s.sorted_id = _lib.ptr(self.sorted_id)
        s.sorted_xyzr = _lib.ptr(self.sorted_xyzr)
        s.scan_partials = _lib.ptr(self.scan_partials)
        s.capacity = cap

    def build(self, population) -> None:
        """Index the active prefix ``[0, count)`` only; query results are global slot indices."""
        if population.device != self.device:
            raise RuntimeError("population and NeighborGrid must live on the same device")
        self.reserve(max(population.capacity, 1))
        with profiling.stage("bin", launches=6):
            _lib.call("wbc_grid_build", ctypes.byref(self._struct), population.count, _lib.ptr(population.position),
                      _lib.ptr(population.radius), _lib.stream(self.device))
        if hasattr(population, "note_spatial_order"):
            population.note_spatial_order(self.sorted_id)

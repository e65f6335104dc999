"""Structure-of-arrays cell storage with preallocated capacity (reference: cells/state.py:31-159).

Slots ``[0, count)`` hold cells (alive or dead), ``[count, capacity)`` are free; daughters are
appended, nothing is reallocated inside the loop and a slot index is a cell's id for life. Every
array is a capacity-sized torch tensor on one CUDA device; the ``active_*`` properties are views
of the prefix.

Randomness: slot i owns the counter-based stream started by ``wbc_rng_init(seed, i)`` for every
slot up to capacity, so results depend on (seed, initial cells) and never on capacity or thread
scheduling. ``rng_state`` holds the uint32 stream states in an int32 tensor (same bits).
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.cells.model import CellState, CellType


@dataclass
class CellPopulation:
    capacity: int
    count: int
    seed: int
    device: torch.device
    position: torch.Tensor  # (capacity, 3) float32, um
    radius: torch.Tensor  # float32, um
    cell_state: torch.Tensor  # int32, CellState
    cell_type: torch.Tensor  # int32, CellType
    age: torch.Tensor  # float32, h
    oxygen_local: torch.Tensor  # float32, mmHg sampled at the cell centre
    glucose_local: torch.Tensor  # float32, mM sampled at the cell centre
    rng_state: torch.Tensor  # int32 bits of the uint32 stream state
    velocity: torch.Tensor  # (capacity, 3) float32, um/h
    neighbor_count: torch.Tensor  # int32
    divide_flag: torch.Tensor  # int32
    division_offset: torch.Tensor  # int32, inclusive prefix sum of divide_flag
    fate_flags: torch.Tensor  # int32
    extra_local: dict = field(default_factory=dict)
    # scratch of commit_divisions: scan partials and the device-side daughter total
    _scan_workspace: torch.Tensor | None = None
    _daughters: torch.Tensor | None = None
    # the hash grid's sorted slot ids of the last binning and the cell count they cover
    _spatial_ids: torch.Tensor | None = None
    _spatial_count: int = -1

    @classmethod
    def from_numpy(
        cls,
        positions: np.ndarray,
        radii: np.ndarray,
        capacity: int | None = None,
        device=None,
        seed: int = 0,
        states: np.ndarray | None = None,
    ) -> CellPopulation:
        positions = np.ascontiguousarray(positions, dtype=np.float32)
        radii = np.ascontiguousarray(radii, dtype=np.float32)
        if positions.ndim != 2 or positions.shape[1] != 3:
            raise ValueError(f"positions must have shape (n, 3), got {positions.shape}")
        count = positions.shape[0]
        if radii.shape != (count,):
            raise ValueError(f"radii must have shape ({count},), got {radii.shape}")
        capacity = count if capacity is None else int(capacity)
        if capacity < count:
            raise ValueError(f"capacity {capacity} smaller than initial cell count {count}")
        if states is None:
            states = np.full(count, int(CellState.PROLIFERATIVE), dtype=np.int32)
        states = np.ascontiguousarray(states, dtype=np.int32)
        if states.shape != (count,):
            raise ValueError(f"states must have shape ({count},), got {states.shape}")
        dev = _lib.resolve_device(device)

        def padded(values, dtype, fill=0):
            buf = np.full((capacity,) + values.shape[1:], fill, dtype=dtype)
            buf[:count] = values
            return torch.from_numpy(buf).to(dev)

        def zeros(*shape, dtype=torch.float32):
            return torch.zeros(shape, dtype=dtype, device=dev)

        pop = cls(
            capacity=capacity,
            count=count,
            seed=int(seed),
            device=dev,
            position=padded(positions, np.float32),
            radius=padded(radii, np.float32),
            cell_state=padded(states, np.int32, fill=int(CellState.DEAD)),
            cell_type=torch.full((capacity,), int(CellType.TUMOR), dtype=torch.int32, device=dev),
            age=zeros(capacity),
            oxygen_local=zeros(capacity),
            glucose_local=zeros(capacity),
            rng_state=zeros(capacity, dtype=torch.int32),
            velocity=zeros(capacity, 3),
            neighbor_count=zeros(capacity, dtype=torch.int32),
            divide_flag=zeros(capacity, dtype=torch.int32),
            division_offset=zeros(capacity, dtype=torch.int32),
            fate_flags=zeros(capacity, dtype=torch.int32),
        )
        # Streams of free slots are initialised too, so a daughter born into slot j draws the
        # same numbers whenever it appears.
        with torch.cuda.device(dev):
            _lib.call("wbc_rng_init", pop.seed, _lib.ptr(pop.rng_state), capacity, _lib.stream(dev))
        return pop

    # ---- scratch -------------------------------------------------------------------------------
    def note_spatial_order(self, sorted_ids: torch.Tensor) -> None:
        """Record the slots in hash-grid order after a binning of the active prefix."""
        self._spatial_ids = sorted_ids
        self._spatial_count = self.count

    def spatial_order(self) -> torch.Tensor | None:
        """The active slots in the order of the last binning (a permutation of [0, count), cells
        that are neighbours in space next to one another), or None when the population changed
        size since; kernels whose result does not depend on the visiting order use it for locality."""
        if self._spatial_ids is None or self._spatial_count != self.count:
            return None
        return self._spatial_ids

    def scan_workspace(self) -> tuple[torch.Tensor, torch.Tensor]:
        """Scan partials (capacity-sized, allocated once) and the int32 daughter total."""
        if self._scan_workspace is None:
            nbytes = int(_lib.load().wbc_scan_workspace_bytes(max(self.capacity, 1)))
            self._scan_workspace = torch.zeros((nbytes + 3) // 4, dtype=torch.int32, device=self.device)
            self._daughters = torch.zeros(1, dtype=torch.int32, device=self.device)
        return self._scan_workspace, self._daughters

    # ---- views over the active prefix ----------------------------------------------------------
    @property
    def active_position(self) -> torch.Tensor:
        return self.position[: self.count]

    @property
    def active_radius(self) -> torch.Tensor:
        return self.radius[: self.count]

    def _np(self, t: torch.Tensor) -> np.ndarray:
        return t[: self.count].cpu().numpy().copy()

    def positions_numpy(self) -> np.ndarray:
        return self._np(self.position)

    def radii_numpy(self) -> np.ndarray:
        return self._np(self.radius)

    def states_numpy(self) -> np.ndarray:
        return self._np(self.cell_state)

    def ages_numpy(self) -> np.ndarray:
        return self._np(self.age)

    def oxygen_numpy(self) -> np.ndarray:
        return self._np(self.oxygen_local)

    def glucose_numpy(self) -> np.ndarray:
        return self._np(self.glucose_local)

    def neighbor_counts_numpy(self) -> np.ndarray:
        return self._np(self.neighbor_count)

    def fate_flags_numpy(self) -> np.ndarray:
        return self._np(self.fate_flags)

    def rng_numpy(self) -> np.ndarray:
        """uint32 stream states of the active prefix."""
        return self._np(self.rng_state).view(np.uint32)

    def local_field(self, name: str) -> torch.Tensor:
        """Per-cell sampled values of a species: oxygen and glucose are first-class, others are
        allocated on first use (capacity-sized)."""
        if name == "oxygen":
            return self.oxygen_local
        if name == "glucose":
            return self.glucose_local
        if name not in self.extra_local:
            self.extra_local[name] = torch.zeros(self.capacity, dtype=torch.float32, device=self.device)
        return self.extra_local[name]

    def local_numpy(self, name: str) -> np.ndarray:
        return self._np(self.local_field(name))

"""State census on the device (reference: metrics/population.py:13-19)."""

from __future__ import annotations

import torch

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.cells.model import CellState


def state_counts(population) -> dict[CellState, int]:
    """Number of cells in each state over the active prefix (one host copy)."""
    counts = torch.zeros(4, dtype=torch.int32, device=population.device)
    if population.count > 0:
        _lib.call("wbc_count_states", population.count, _lib.ptr(population.cell_state), _lib.ptr(counts),
                  _lib.stream(population.device))
    values = counts.cpu().numpy()
    return {state: int(values[int(state)]) for state in CellState}

"""Cell states and types (reference: cells/model.py:14-22).

``cell_state`` is the single source of truth for a cell's condition, with the precedence
DEAD > HYPOXIC > QUIESCENT > PROLIFERATIVE. The integer values are shared with the kernels.
"""

from enum import IntEnum


class CellState(IntEnum):
    PROLIFERATIVE = 0
    QUIESCENT = 1
    HYPOXIC = 2
    DEAD = 3


class CellType(IntEnum):
    TUMOR = 0


STATE_PROLIFERATIVE = int(CellState.PROLIFERATIVE)
STATE_QUIESCENT = int(CellState.QUIESCENT)
STATE_HYPOXIC = int(CellState.HYPOXIC)
STATE_DEAD = int(CellState.DEAD)
NUM_STATES = len(CellState)

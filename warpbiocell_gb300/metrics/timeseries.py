"""Onsets of hypoxia and necrosis in a run's metrics rows (the onset columns of a sweep summary;
reference: metrics/timeseries.py, whose function names and column names these keep).

A run records one row per observation (time, cell counts per state, spheroid radius, ...). The
onset of a condition is the first observation at which its cell count is positive; it is reported
as the time and the spheroid radius of that row, or NaN for both when it never happens.
"""

from __future__ import annotations

import math

# (label of the summary columns, count column whose first positive value marks the onset)
ONSET_CONDITIONS = (("hypoxia", "hypoxic_cells"), ("necrosis", "dead_cells"))


def onset(rows: list[dict], column: str, radius_column: str = "spheroid_radius_um") -> tuple[float, float]:
    """(time_h, radius) of the first row with ``column`` > 0, or (NaN, NaN)."""
    first = next((row for row in rows if float(row[column]) > 0.0), None)
    if first is None:
        return math.nan, math.nan
    return float(first["time_h"]), float(first[radius_column])


def onset_summary(rows: list[dict]) -> dict[str, float]:
    """``<label>_onset_time_h`` and ``<label>_onset_radius_um`` for hypoxia and necrosis."""
    summary: dict[str, float] = {}
    for label, column in ONSET_CONDITIONS:
        time_h, radius = onset(rows, column)
        summary[f"{label}_onset_time_h"] = time_h
        summary[f"{label}_onset_radius_um"] = radius
    return summary

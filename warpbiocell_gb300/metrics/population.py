"""Population metrics (reference: metrics/population.py): the state census runs on the device
(one host copy of four counts); the geometric summaries and radial profiles are computed on host
copies of the positions, as the reference does."""

from __future__ import annotations

import numpy as np
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


def population_summary(population, oxygen=None) -> dict[str, float]:
    """Counts, the 99th-percentile distance from the centroid (the spheroid radius), the mean cell
    radius and, with fields, their values at living cells and over the grid (reference:
    metrics/population.py:22-46)."""
    counts = state_counts(population)
    x = population.positions_numpy()
    dist = np.linalg.norm(x - x.mean(axis=0), axis=1) if x.shape[0] else np.zeros(0)
    summary = {
        "cells": population.count,
        "living_cells": population.count - counts[CellState.DEAD],
        "dead_cells": counts[CellState.DEAD],
        "proliferative_cells": counts[CellState.PROLIFERATIVE],
        "quiescent_cells": counts[CellState.QUIESCENT],
        "hypoxic_cells": counts[CellState.HYPOXIC],
        "spheroid_radius": float(np.percentile(dist, 99)) if dist.size else 0.0,
        "mean_radius": float(population.radii_numpy().mean()) if population.count else 0.0,
    }
    if oxygen is not None:
        summary.update(oxygen_summary(population, oxygen))
        summary.update(species_summary(population, oxygen))
    return summary


def oxygen_summary(population, oxygen) -> dict[str, float]:
    """Oxygen at living cells and over the updated grid nodes [mmHg] (OxygenField or MetabolicFields)."""
    alive = population.states_numpy() != int(CellState.DEAD)
    at_cells = population.oxygen_numpy()[alive]
    grid = oxygen.numpy()[oxygen.field.interior_mask()]
    report = oxygen.last_report
    return {
        "oxygen_cells_mean": float(at_cells.mean()) if at_cells.size else float("nan"),
        "oxygen_cells_min": float(at_cells.min()) if at_cells.size else float("nan"),
        "oxygen_grid_mean": float(grid.mean()),
        "oxygen_grid_min": float(grid.min()),
        "field_sweeps": report.sweeps if report else 0,
    }


def species_summary(population, fields) -> dict[str, float]:
    """Mean / min / max at living cells of every species beyond oxygen."""
    names = [n for n in getattr(fields, "names", []) if n != "oxygen"]
    if not names:
        return {}
    alive = population.states_numpy() != int(CellState.DEAD)
    out = {}
    for name in names:
        values = population.local_numpy(name)[alive]
        for stat, fn in (("mean", np.mean), ("min", np.min), ("max", np.max)):
            out[f"{name}_cells_{stat}"] = float(fn(values)) if values.size else float("nan")
    return out


def radial_profile(population, n_bins: int | None = None, shell_width: float | None = None) -> dict[str, np.ndarray]:
    """Mean oxygen (glucose, lactate) and state fractions in shells around the centroid: ``n_bins``
    equal shells up to the outermost cell, or shells of fixed ``shell_width`` [um]."""
    x = population.positions_numpy()
    r = np.linalg.norm(x - x.mean(axis=0), axis=1) if x.shape[0] else np.zeros(0)
    r_max = float(r.max()) if r.size else 0.0
    if shell_width is not None:
        n_bins = max(1, int(np.ceil((r_max + 1e-6) / shell_width)))
        edges = shell_width * np.arange(n_bins + 1)
    else:
        n_bins = n_bins or 10
        edges = np.linspace(0.0, r_max + 1e-6, n_bins + 1)
    which = np.minimum(np.digitize(r, edges) - 1, n_bins - 1)
    cells = np.bincount(which, minlength=n_bins)

    def shell_mean(values):
        sums = np.bincount(which, weights=values.astype(np.float64), minlength=n_bins)
        with np.errstate(invalid="ignore", divide="ignore"):
            return np.where(cells > 0, sums / np.maximum(cells, 1), np.nan)

    out = {"r_outer": edges[1:], "cells": cells, "oxygen_mean": shell_mean(population.oxygen_numpy())}
    for name in ("glucose", "lactate"):
        if name == "glucose" or name in population.extra_local:
            out[f"{name}_mean"] = shell_mean(population.local_numpy(name))
    states = population.states_numpy()
    for state in CellState:
        out[f"fraction_{state.name.lower()}"] = shell_mean((states == int(state)).astype(np.float64))
    return out


def shell_radii(profile: dict[str, np.ndarray]) -> dict[str, float]:
    """Outer edge [um] of the outermost shell where dead / hypoxic-or-dead / non-proliferative
    cells are at least half; 0 when none."""

    def outermost(fraction):
        hit = np.where(np.nan_to_num(fraction) >= 0.5)[0]
        return float(profile["r_outer"][hit.max()]) if hit.size else 0.0

    dead = profile["fraction_dead"]
    return {
        "necrotic_radius": outermost(dead),
        "hypoxic_radius": outermost(profile["fraction_hypoxic"] + dead),
        "non_proliferative_radius": outermost(1.0 - profile["fraction_proliferative"]),
    }

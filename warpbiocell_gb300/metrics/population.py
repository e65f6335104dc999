"""Population metrics (reference: metrics/population.py, whose function names, dictionary keys and
definitions these keep): the state census, the spheroid's size, the fields at the living cells
and radial shell profiles.

Everything is reduced on the device from the population's arrays, and each function copies one
small vector of results to the host (the state census runs in the library's counting kernel).
Definitions: the spheroid radius is the 99th percentile (linear interpolation) of the cells'
distances from their centroid; field statistics at cells are over living cells only; grid
statistics are over the nodes the solver updates; a radial profile bins cells by distance from
the centroid into shells that end at the outermost cell or have a fixed width.
"""

from __future__ import annotations

import numpy as np
import torch

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.cells.model import CellState

_NAN = float("nan")


def state_counts(population) -> dict[CellState, int]:
    """Number of cells in each state over the active prefix (one host copy)."""
    counts = torch.zeros(4, dtype=torch.int32, device=population.device)
    if population.count > 0:
        _lib.call("wbc_count_states", population.count, _lib.ptr(population.cell_state), _lib.ptr(counts),
                  _lib.stream(population.device))
    values = counts.cpu().tolist()
    return {state: int(values[int(state)]) for state in CellState}


def _distances(population) -> torch.Tensor:
    """Distances [um] of the active cells from their centroid (float64, on the device)."""
    x = population.position[: population.count].double()
    if x.shape[0] == 0:
        return x.new_zeros(0)
    return torch.linalg.vector_norm(x - x.mean(dim=0), dim=1)


def _percentile(values: torch.Tensor, q: float) -> torch.Tensor:
    """The q-th percentile with linear interpolation between order statistics (numpy's default)."""
    ordered = torch.sort(values).values
    at = q / 100.0 * (ordered.numel() - 1)
    lo = int(np.floor(at))
    hi = min(lo + 1, ordered.numel() - 1)
    return ordered[lo] + (ordered[hi] - ordered[lo]) * (at - lo)


def _living(population) -> torch.Tensor:
    return population.cell_state[: population.count] != int(CellState.DEAD)


def population_summary(population, oxygen=None) -> dict[str, float]:
    """Counts per state, the spheroid radius, the mean cell radius and, given the fields, their
    values at living cells and over the grid (reference: metrics/population.py:22-46)."""
    counts = state_counts(population)
    n = population.count
    summary = {
        "cells": n,
        "living_cells": n - counts[CellState.DEAD],
        "dead_cells": counts[CellState.DEAD],
        "proliferative_cells": counts[CellState.PROLIFERATIVE],
        "quiescent_cells": counts[CellState.QUIESCENT],
        "hypoxic_cells": counts[CellState.HYPOXIC],
        "spheroid_radius": 0.0,
        "mean_radius": 0.0,
    }
    if n:
        size = torch.stack([_percentile(_distances(population), 99.0),
                            population.radius[:n].double().mean()]).cpu().tolist()
        summary["spheroid_radius"], summary["mean_radius"] = size
    if oxygen is not None:
        summary.update(oxygen_summary(population, oxygen))
        summary.update(species_summary(population, oxygen))
    return summary


def _stats_at(values: torch.Tensor, mask: torch.Tensor, kinds: tuple[str, ...]) -> list[torch.Tensor]:
    picked = values[mask].double()
    if picked.numel() == 0:
        return [torch.tensor(_NAN, dtype=torch.float64, device=values.device) for _ in kinds]
    reducers = {"mean": torch.mean, "min": torch.min, "max": torch.max}
    return [reducers[k](picked) for k in kinds]


def oxygen_summary(population, oxygen) -> dict[str, float]:
    """Oxygen [mmHg] at living cells and over the updated grid nodes (OxygenField or MetabolicFields)."""
    n = population.count
    cells = _stats_at(population.oxygen_local[:n], _living(population), ("mean", "min"))
    field = oxygen.field
    grid = _stats_at(field.values, field.interior_mask_tensor(), ("mean", "min"))
    values = torch.stack(cells + grid).cpu().tolist()
    report = oxygen.last_report
    return {"oxygen_cells_mean": values[0], "oxygen_cells_min": values[1], "oxygen_grid_mean": values[2],
            "oxygen_grid_min": values[3], "field_sweeps": report.sweeps if report else 0}


def species_summary(population, fields) -> dict[str, float]:
    """Mean, min and max at living cells of every species other than oxygen."""
    names = [name for name in getattr(fields, "names", []) if name != "oxygen"]
    if not names:
        return {}
    kinds = ("mean", "min", "max")
    living = _living(population)
    stats = []
    for name in names:
        stats += _stats_at(population.local_field(name)[: population.count], living, kinds)
    values = torch.stack(stats).cpu().tolist()
    keys = [f"{name}_cells_{kind}" for name in names for kind in kinds]
    return dict(zip(keys, values))


def radial_profile(population, n_bins: int | None = None, shell_width: float | None = None) -> dict[str, np.ndarray]:
    """Mean oxygen (glucose, lactate) and state fractions in shells around the centroid: ``n_bins``
    equal shells up to just beyond the outermost cell (10 by default), or shells of fixed
    ``shell_width`` [um] covering it."""
    dist = _distances(population)
    r_max = float(dist.max()) if dist.numel() else 0.0
    if shell_width is not None:
        n_bins = max(1, int(np.ceil((r_max + 1e-6) / shell_width)))
        edges = shell_width * np.arange(n_bins + 1)
    else:
        n_bins = n_bins or 10
        edges = np.linspace(0.0, r_max + 1e-6, n_bins + 1)
    dev = population.device
    # shell of each cell: edges[b] <= r < edges[b + 1], the last shell open above
    shell = torch.clamp(torch.bucketize(dist, torch.as_tensor(edges, device=dev), right=True) - 1, max=n_bins - 1)
    members = torch.bincount(shell, minlength=n_bins).double()

    def shell_mean(values: torch.Tensor) -> torch.Tensor:
        sums = torch.zeros(n_bins, dtype=torch.float64, device=dev).index_add_(0, shell, values.double())
        return torch.where(members > 0, sums / members.clamp(min=1.0), torch.full_like(sums, _NAN))

    n = population.count
    columns = {"oxygen_mean": shell_mean(population.oxygen_local[:n])}
    for name in ("glucose", "lactate"):
        if name == "glucose" or name in population.extra_local:
            columns[f"{name}_mean"] = shell_mean(population.local_field(name)[:n])
    states = population.cell_state[:n]
    for state in CellState:
        columns[f"fraction_{state.name.lower()}"] = shell_mean(states == int(state))
    host = {key: value.cpu().numpy() for key, value in columns.items()}
    return {"r_outer": edges[1:], "cells": members.cpu().numpy().astype(np.int64), **host}


def shell_radii(profile: dict[str, np.ndarray]) -> dict[str, float]:
    """Outer edge [um] of the outermost shell in which dead, hypoxic-or-dead, and
    non-proliferative cells respectively make up at least half of the cells (0 if no shell does)."""
    outer = np.asarray(profile["r_outer"], dtype=float)
    dead = np.asarray(profile["fraction_dead"])
    criteria = {"necrotic_radius": dead,
                "hypoxic_radius": np.asarray(profile["fraction_hypoxic"]) + dead,
                "non_proliferative_radius": 1.0 - np.asarray(profile["fraction_proliferative"])}
    radii = {}
    for key, fraction in criteria.items():
        majority = np.flatnonzero(np.nan_to_num(fraction) >= 0.5)
        radii[key] = float(outer[majority[-1]]) if majority.size else 0.0
    return radii

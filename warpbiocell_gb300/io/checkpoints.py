"""Checkpoints: every persistent cell array plus the fields, as a compressed ``.npz``
(reference: io/checkpoints.py:16-45, same keys and dtypes: ``rng_state`` as uint32 stream
states, ``network_states`` as uint64 words).

Beyond the reference's keys a checkpoint carries ``neighbor_count`` (the contact counts the last
mechanics substep left for the next lifecycle decision), which makes :func:`restore_population`
plus :func:`restore_fields` / :func:`restore_network` continue a run bit for bit: the free slots'
random streams are re-initialised from the seed exactly as at the start of the run, so a daughter
born after the restart draws what it would have drawn without it.
"""

from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

from warpbiocell_gb300.cells.state import CellPopulation

CELL_ARRAYS = ("position", "radius", "cell_state", "cell_type", "age", "oxygen_local", "glucose_local", "fate_flags",
               "rng_state")


def _host(t: torch.Tensor, n: int) -> np.ndarray:
    return t[:n].detach().cpu().numpy().copy()


def save_checkpoint(path: str | Path, population: CellPopulation, oxygen, time_h: float, region=None,
                    network=None) -> Path:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    n = population.count
    arrays = {name: _host(getattr(population, name), n) for name in CELL_ARRAYS}
    arrays["rng_state"] = arrays["rng_state"].view(np.uint32)
    arrays["neighbor_count"] = _host(population.neighbor_count, n)
    arrays["count"] = np.array(n)
    arrays["capacity"] = np.array(population.capacity)
    arrays["seed"] = np.array(population.seed)
    arrays["time_h"] = np.array(time_h)
    for name, values in population.extra_local.items():
        arrays[f"{name}_local"] = _host(values, n)
    if oxygen is not None:
        fields = getattr(oxygen, "species_fields", None) or {"oxygen": oxygen}
        for name, species in fields.items():
            arrays["field" if name == "oxygen" else f"field_{name}"] = species.numpy()
        arrays["density"] = fields["oxygen"].density.detach().cpu().numpy()
        arrays["grid_origin"] = np.array(oxygen.geometry.origin)
        arrays["grid_dx"] = np.array(oxygen.geometry.dx)
    if region is not None:
        arrays["tissue_sdf"] = region.sdf_numpy()
        arrays["grid_origin"] = np.array(region.geometry.origin)
        arrays["grid_dx"] = np.array(region.geometry.dx)
    if network is not None:
        arrays["network_states"] = _host(network.states, n).view(np.uint64)
        arrays["network_nodes"] = np.array(network.network.names)
    np.savez_compressed(path, **arrays)
    return path


def load_checkpoint(path: str | Path) -> dict[str, np.ndarray]:
    with np.load(Path(path)) as data:
        return {key: data[key] for key in data.files}


def restore_population(data: dict, capacity: int | None = None, device=None) -> CellPopulation:
    """A population holding the checkpoint's cells (capacity defaults to the checkpoint's)."""
    n = int(data["count"])
    capacity = int(data["capacity"]) if capacity is None else int(capacity)
    pop = CellPopulation.from_numpy(data["position"].reshape(n, 3), data["radius"], capacity=capacity, device=device,
                                    seed=int(data["seed"]), states=data["cell_state"])
    for name in ("cell_type", "age", "oxygen_local", "glucose_local", "fate_flags"):
        getattr(pop, name)[:n].copy_(torch.from_numpy(np.ascontiguousarray(data[name])))
    pop.rng_state[:n].copy_(torch.from_numpy(np.ascontiguousarray(data["rng_state"]).view(np.int32)))
    if "neighbor_count" in data:
        pop.neighbor_count[:n].copy_(torch.from_numpy(np.ascontiguousarray(data["neighbor_count"])))
    for key, values in data.items():
        if key.endswith("_local") and key not in ("oxygen_local", "glucose_local"):
            pop.local_field(key[: -len("_local")])[:n].copy_(torch.from_numpy(np.ascontiguousarray(values)))
    return pop


def restore_fields(data: dict, oxygen) -> None:
    """Put the checkpoint's field values back (the warm start of the next solve)."""
    fields = getattr(oxygen, "species_fields", None) or {"oxygen": oxygen}
    for name, species in fields.items():
        key = "field" if name == "oxygen" else f"field_{name}"
        if key not in data:
            raise KeyError(f"checkpoint has no {key!r}")
        species.field.values.copy_(torch.from_numpy(np.ascontiguousarray(data[key], dtype=np.float32)))


def restore_network(data: dict, network, population: CellPopulation) -> None:
    names = [str(x) for x in data["network_nodes"]]
    if names != list(network.network.names):
        raise ValueError("checkpoint network nodes differ from the runtime's network")
    n = population.count
    words = np.ascontiguousarray(data["network_states"]).view(np.int64)
    network.states[:n].copy_(torch.from_numpy(words.reshape(n, -1)))

"""The checkpoint file format on the host (no device): the keys, shapes and dtypes the reference's
writer produces (reference: io/checkpoints.py:16-45; ``rng_state`` as uint32 stream states,
``network_states`` as uint64 words), plus ``neighbor_count``, which makes a resumed run continue
bit for bit. The population here holds host tensors, built field by field."""

from types import SimpleNamespace

import numpy as np
import torch

from warpbiocell_gb300.cells.state import CellPopulation
from warpbiocell_gb300.io.checkpoints import CELL_ARRAYS, load_checkpoint, save_checkpoint

# The arrays the reference writes for a population with a field and a network (io/checkpoints.py).
REFERENCE_KEYS = {"position", "radius", "cell_state", "cell_type", "age", "oxygen_local", "glucose_local",
                  "fate_flags", "rng_state", "count", "capacity", "seed", "time_h", "field", "density",
                  "grid_origin", "grid_dx", "network_states", "network_nodes"}


def _host_population(n: int, capacity: int) -> CellPopulation:
    rng = np.random.default_rng(5)

    def f32(*shape):
        return torch.from_numpy(rng.random(shape, dtype=np.float32))

    def i32(lo, hi):
        return torch.from_numpy(rng.integers(lo, hi, capacity, dtype=np.int32))

    return CellPopulation(
        capacity=capacity, count=n, seed=11, device=torch.device("cpu"),
        position=f32(capacity, 3), radius=f32(capacity), cell_state=i32(0, 4), cell_type=i32(0, 2),
        age=f32(capacity), oxygen_local=f32(capacity), glucose_local=f32(capacity),
        rng_state=i32(-2**31, 2**31 - 1), velocity=f32(capacity, 3), neighbor_count=i32(0, 30),
        divide_flag=i32(0, 2), division_offset=i32(0, 9), fate_flags=i32(0, 16))


def _fields(shape=(5, 6, 7)):
    values = np.arange(np.prod(shape), dtype=np.float32).reshape(shape)
    return SimpleNamespace(geometry=SimpleNamespace(origin=(-1.0, -2.0, -3.0), dx=2.5), numpy=lambda: values.copy(),
                           density=torch.ones(shape), species_fields=None)


def test_checkpoint_keys_shapes_and_dtypes_match_the_reference(tmp_path):
    n, capacity = 6, 10
    pop = _host_population(n, capacity)
    words = torch.from_numpy(np.random.default_rng(2).integers(-2**63, 2**63 - 1, (capacity, 2), dtype=np.int64))
    network = SimpleNamespace(states=words, network=SimpleNamespace(names=["A", "B", "Proliferation"]))
    path = save_checkpoint(tmp_path / "c" / "state.npz", pop, _fields(), 1.5, network=network)
    data = load_checkpoint(path)

    assert set(data) == REFERENCE_KEYS | {"neighbor_count"}
    assert set(CELL_ARRAYS) <= set(data)
    assert data["position"].shape == (n, 3) and data["position"].dtype == np.float32
    for name in ("radius", "age", "oxygen_local", "glucose_local"):
        assert data[name].shape == (n,) and data[name].dtype == np.float32
    for name in ("cell_state", "cell_type", "fate_flags", "neighbor_count"):
        assert data[name].shape == (n,) and data[name].dtype == np.int32
        np.testing.assert_array_equal(data[name], getattr(pop, name)[:n].numpy())
    # stream states: the same 32 bits, read as unsigned
    assert data["rng_state"].dtype == np.uint32
    np.testing.assert_array_equal(data["rng_state"].view(np.int32), pop.rng_state[:n].numpy())
    # node states: the same 64-bit words, read as unsigned
    assert data["network_states"].dtype == np.uint64 and data["network_states"].shape == (n, 2)
    np.testing.assert_array_equal(data["network_states"].view(np.int64), words[:n].numpy())
    assert list(data["network_nodes"]) == ["A", "B", "Proliferation"]
    assert (int(data["count"]), int(data["capacity"]), int(data["seed"])) == (n, capacity, 11)
    assert float(data["time_h"]) == 1.5
    assert data["field"].shape == (5, 6, 7) and data["density"].shape == (5, 6, 7)
    np.testing.assert_array_equal(data["grid_origin"], [-1.0, -2.0, -3.0])
    assert float(data["grid_dx"]) == 2.5


def test_checkpoint_carries_extra_species_and_their_cell_samples(tmp_path):
    pop = _host_population(4, 4)
    pop.extra_local["lactate"] = torch.arange(4, dtype=torch.float32)
    oxygen, lactate = _fields(), _fields()
    metabolic = SimpleNamespace(geometry=oxygen.geometry, species_fields={"oxygen": oxygen, "lactate": lactate})
    data = load_checkpoint(save_checkpoint(tmp_path / "s.npz", pop, metabolic, 0.0))
    assert {"field", "field_lactate", "lactate_local", "density"} <= set(data)
    np.testing.assert_array_equal(data["lactate_local"], [0.0, 1.0, 2.0, 3.0])
    assert "network_states" not in data and "tissue_sdf" not in data

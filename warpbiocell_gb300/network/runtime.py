"""Per-cell Boolean networks on the device: parameters, state arrays and the per-step update
(reference: network/runtime.py:89-228).

Order inside a cell step: ``clamp_inputs`` sets the input nodes from the sampled fields,
``update`` advances every cell's network (all synchronous sweeps of a step in one launch, the
words held in registers), ``read_fates`` packs the fate nodes into ``population.fate_flags``;
after division ``inherit`` copies the parent's words to the daughter.

``states`` is a ``(capacity, n_words)`` int64 tensor holding the uint64 words (same bits).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.network.model import BooleanNetwork, NetworkError

FATE_PROLIFERATION, FATE_APOPTOSIS, FATE_GROWTH_ARREST, FATE_NECROSIS = 1, 2, 4, 8
SOURCES = {"oxygen": 0, "glucose": 1, "constant": 4}  # other species: extra_a (2), extra_b (3)
UPDATE_MODES = ("asynchronous", "synchronous", "maboss")
FATE_BITS = {"proliferation": FATE_PROLIFERATION, "apoptosis": FATE_APOPTOSIS, "growth_arrest": FATE_GROWTH_ARREST,
             "necrosis": FATE_NECROSIS}
FATE_ROLES = tuple(FATE_BITS)
DEFAULT_OUTPUT_NODES = {"proliferation": "Proliferation", "apoptosis": "Apoptosis", "growth_arrest": "Growth_Arrest",
                        "necrosis": "Necrosis"}


@dataclass(frozen=True)
class InputClamp:
    """Input node driven by the environment: ``source`` is oxygen, glucose, a species name, or
    constant; ON when the value is above (or, with ``above=False``, below) ``threshold``; for
    ``constant`` ON when ``threshold > 0``."""

    node: str
    source: str
    threshold: float = 0.0
    above: bool = True


@dataclass(frozen=True)
class NetworkParams:
    network: BooleanNetwork
    update: str = "asynchronous"
    updates_per_step: int = 100
    time_units_per_h: float = 10.0
    max_events_per_step: int = 20000
    inputs: tuple = ()
    outputs: dict | None = None
    initial_states: dict = field(default_factory=dict)

    def __post_init__(self):
        if self.update not in UPDATE_MODES:
            raise NetworkError(f"update must be one of {UPDATE_MODES}, got {self.update!r}")
        if self.updates_per_step < 1 or self.time_units_per_h <= 0.0 or self.max_events_per_step < 1:
            raise NetworkError("updates_per_step, time_units_per_h and max_events_per_step must be positive")
        names = set(self.network.index)
        for clamp in self.inputs:
            if clamp.node not in names:
                raise NetworkError(f"input clamp refers to unknown node {clamp.node!r}")
        if self.outputs is None:
            object.__setattr__(self, "outputs",
                               {role: (node if node in names else None) for role, node in DEFAULT_OUTPUT_NODES.items()})
        for role, name in self.outputs.items():
            if role not in FATE_BITS:
                raise NetworkError(f"unknown output role {role!r}; use {sorted(FATE_BITS)}")
            if name is not None and name not in names:
                raise NetworkError(f"output {role!r} refers to unknown node {name!r}")
        for name in self.initial_states:
            if name not in names:
                raise NetworkError(f"initial_states refers to unknown node {name!r}")

    def fate_node_indices(self) -> tuple[int, int, int, int]:
        idx = self.network.index
        return tuple(idx[self.outputs[role]] if self.outputs.get(role) else -1 for role in FATE_ROLES)


class NetworkRuntime:
    def __init__(self, params: NetworkParams, capacity: int, device=None, species_names: tuple[str, ...] = ()):
        self.params = params
        self.network = params.network
        self.device = _lib.resolve_device(device)
        self.capacity = capacity
        arrays = self.network.programs()
        p_on = arrays["p_on"].copy()
        for name, p in params.initial_states.items():
            p_on[self.network.index[name]] = float(p)
        arrays["p_on"] = p_on
        self._arrays = {k: torch.from_numpy(np.ascontiguousarray(v)).to(self.device) for k, v in arrays.items()}
        self.states = torch.zeros((capacity, self.network.n_words), dtype=torch.int64, device=self.device)
        self._fate_query = torch.tensor(self.fate_nodes, dtype=torch.int32, device=self.device)
        self._fate_counts = torch.zeros(4, dtype=torch.int32, device=self.device)
        self.species_names = tuple(species_names)
        a = self._arrays
        # Truth tables of the nodes with at most 6 inputs (the kernels evaluate those by lookup,
        # the others by running their programs; both give the program's value).
        tables = self.network.truth_tables(arrays)
        self._tables = {"arity": torch.from_numpy(tables["arity"]).to(self.device),
                        "inputs": torch.from_numpy(tables["inputs"]).to(self.device),
                        "bits": torch.from_numpy(tables["bits"].view(np.int64)).to(self.device)}
        t = self._tables
        self._program = _lib.NetworkProgramC(
            n_nodes=self.network.n_nodes, n_words=self.network.n_words, n_ops=int(a["ops"].numel()),
            n_updatable=int(a["updatable"].numel()), ops=_lib.ptr(a["ops"]), args=_lib.ptr(a["args"]),
            start=_lib.ptr(a["start"]), length=_lib.ptr(a["length"]),
            updatable=_lib.ptr(a["updatable"]) if a["updatable"].numel() else None,
            table_arity=_lib.ptr(t["arity"]), table_inputs=_lib.ptr(t["inputs"]), table_bits=_lib.ptr(t["bits"]))
        self._build_clamps()

    # ---- input mapping -----------------------------------------------------------------------
    def _build_clamps(self) -> None:
        extra = [n for n in self.species_names if n not in ("oxygen", "glucose")]
        nodes, sources, thresholds, above = [], [], [], []
        for clamp in self.params.inputs:
            if clamp.source in SOURCES:
                source = SOURCES[clamp.source]
            elif clamp.source in extra[:2]:
                source = 2 + extra.index(clamp.source)
            else:
                raise NetworkError(f"input clamp {clamp.node!r}: source {clamp.source!r} is not oxygen, glucose, "
                                   f"constant or one of the first two extra species {extra[:2]}")
            nodes.append(self.network.index[clamp.node])
            sources.append(source)
            thresholds.append(float(clamp.threshold))
            above.append(1 if clamp.above else 0)
        self.extra_names = extra[:2]
        dev = self.device
        self._clamp = {
            "node": torch.tensor(nodes or [0], dtype=torch.int32, device=dev),
            "source": torch.tensor(sources or [4], dtype=torch.int32, device=dev),
            "threshold": torch.tensor(np.array(thresholds or [0.0], dtype=np.float32), device=dev),
            "above": torch.tensor(above or [1], dtype=torch.int32, device=dev),
        }
        self._n_clamps = len(nodes)

    @property
    def program(self) -> _lib.NetworkProgramC:
        return self._program

    # ---- per-step operations ---------------------------------------------------------------
    def initialize(self, population, count: int | None = None) -> None:
        """Random initial states for slots [0, count) from the cells' streams."""
        n = population.count if count is None else count
        if n > 0:
            _lib.call("wbc_network_initialize", ctypes.byref(self._program), n, _lib.ptr(self._arrays["p_on"]),
                      _lib.ptr(population.rng_state), _lib.ptr(self.states), _lib.stream(self.device))
            self.read_fates(population)

    def clamp_inputs(self, population) -> None:
        n = population.count
        if n == 0 or self._n_clamps == 0:
            return
        extra_a = population.local_field(self.extra_names[0]) if len(self.extra_names) > 0 else population.oxygen_local
        extra_b = population.local_field(self.extra_names[1]) if len(self.extra_names) > 1 else population.oxygen_local
        c = self._clamp
        _lib.call("wbc_network_clamp_inputs", n, self.network.n_words, self._n_clamps, _lib.ptr(c["node"]),
                  _lib.ptr(c["source"]), _lib.ptr(c["threshold"]), _lib.ptr(c["above"]),
                  _lib.ptr(population.oxygen_local), _lib.ptr(population.glucose_local), _lib.ptr(extra_a),
                  _lib.ptr(extra_b), _lib.ptr(self.states), _lib.stream(self.device))

    def update(self, population, dt_h: float, updates_per_step: int | None = None,
               time_units_per_h: float | None = None) -> None:
        """Advance every cell's network by one cell step of ``dt_h``; the amount of network time
        comes from ``params`` unless overridden here; the mode is fixed at construction."""
        n = population.count
        if n == 0:
            return
        picks = self.params.updates_per_step if updates_per_step is None else int(updates_per_step)
        units = self.params.time_units_per_h if time_units_per_h is None else float(time_units_per_h)
        if picks < 1 or units <= 0.0:
            raise NetworkError("updates_per_step must be >= 1 and time_units_per_h > 0")
        prog = ctypes.byref(self._program)
        s = _lib.stream(self.device)
        if self.params.update == "asynchronous":
            _lib.call("wbc_network_update_async", prog, n, picks, _lib.ptr(population.rng_state),
                      _lib.ptr(self.states), s)
        elif self.params.update == "synchronous":
            _lib.call("wbc_network_update_sync", prog, n, picks, _lib.ptr(self.states), s)
        else:
            a = self._arrays
            _lib.call("wbc_network_update_maboss", prog, n, float(dt_h * units), self.params.max_events_per_step,
                      _lib.ptr(a["rate_up_true"]), _lib.ptr(a["rate_up_false"]), _lib.ptr(a["rate_down_true"]),
                      _lib.ptr(a["rate_down_false"]), _lib.ptr(population.rng_state), _lib.ptr(self.states), s)

    def read_fates(self, population) -> None:
        n = population.count
        if n == 0:
            return
        _lib.call("wbc_network_read_fates", n, self.network.n_words, *self.fate_nodes, _lib.ptr(self.states),
                  _lib.ptr(population.fate_flags), _lib.stream(self.device))

    @property
    def fate_nodes(self) -> tuple[int, int, int, int]:
        return self.params.fate_node_indices()

    def inherit(self, population, count_before: int) -> None:
        """After a lifecycle step that created daughters: copy parents' networks to them."""
        if count_before == 0 or population.count == count_before:
            return
        _lib.call("wbc_network_inherit", count_before, self.network.n_words, _lib.ptr(population.divide_flag),
                  _lib.ptr(population.division_offset), _lib.ptr(self.states), _lib.stream(self.device))

    def step(self, population, dt_h: float) -> None:
        """clamp -> update -> fates, the per-cell-step sequence."""
        self.clamp_inputs(population)
        self.update(population, dt_h)
        self.read_fates(population)

    # ---- inspection --------------------------------------------------------------------------
    def words_numpy(self, population) -> np.ndarray:
        """uint64 words of the active prefix, (count, n_words)."""
        return self.states[: population.count].cpu().numpy().view(np.uint64).copy()

    def states_numpy(self, population) -> np.ndarray:
        """Boolean matrix (count, n_nodes)."""
        words = self.states[: population.count].cpu().numpy()
        bits = np.unpackbits(np.ascontiguousarray(words).view(np.uint8).reshape(population.count, -1), axis=1,
                             bitorder="little")
        return bits[:, : self.network.n_nodes].astype(bool)

    def count_on(self, population, names: list[str], living_only: bool = True) -> np.ndarray:
        nodes = torch.tensor([self.network.index[n] for n in names], dtype=torch.int32, device=self.device)
        counts = torch.zeros(len(names), dtype=torch.int32, device=self.device)
        if population.count > 0:
            _lib.call("wbc_network_count_on", population.count, self.network.n_words, len(names), _lib.ptr(nodes),
                      1 if living_only else 0, _lib.ptr(population.cell_state), _lib.ptr(self.states),
                      _lib.ptr(counts), _lib.stream(self.device))
        return counts.cpu().numpy()

    def fate_counts(self, population) -> dict[str, int]:
        self._fate_counts.zero_()
        if population.count > 0:
            _lib.call("wbc_network_count_on", population.count, self.network.n_words, 4, _lib.ptr(self._fate_query),
                      1, _lib.ptr(population.cell_state), _lib.ptr(self.states), _lib.ptr(self._fate_counts),
                      _lib.stream(self.device))
        values = self._fate_counts.cpu().numpy()
        return {role: int(values[k]) for k, role in enumerate(FATE_ROLES)}

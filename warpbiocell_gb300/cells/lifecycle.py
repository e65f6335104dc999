"""Cell lifecycle step: death, hypoxia, contact inhibition and division with deterministic slot
allocation (reference: cells/lifecycle.py:14-187).

``decide_lifecycle`` launches ``wbc_lifecycle_decide`` (no host sync). ``commit_divisions`` runs
the inclusive prefix sum of ``divide_flag`` on the device (``wbc_division_scan``), reads the
daughter total once (the single host sync of a cell step, as in the reference), checks the
capacity, then ``wbc_place_daughters`` writes daughter k of the step into slot count + k.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

from warpbiocell_gb300 import _lib, profiling


class CapacityError(RuntimeError):
    """Raised when a step would create more cells than the population was allocated for."""


@dataclass(frozen=True)
class LifecycleParams:
    """Stochastic, rate-based lifecycle (units: rates 1/h, oxygen mmHg, glucose mM); the field
    meanings and defaults are those of the reference's LifecycleParams."""

    division_rate: float = 0.0289
    death_rate: float = 0.0
    anoxic_death_rate: float = 0.0
    inhibition_threshold: int = 8
    hypoxia_threshold: float = 0.0
    death_threshold: float = 0.0
    glucose_threshold: float = 0.0
    glucose_death_threshold: float = 0.0
    necrosis_requires_glucose: bool = False
    placement_factor: float = 1.0
    phenotype_model: str = "rules"
    apoptosis_rate: float = 0.0
    necrosis_rate: float = 0.0

    def __post_init__(self):
        if self.division_rate < 0.0 or self.death_rate < 0.0 or self.anoxic_death_rate < 0.0:
            raise ValueError("rates must be non-negative")
        if self.apoptosis_rate < 0.0 or self.necrosis_rate < 0.0:
            raise ValueError("apoptosis_rate and necrosis_rate must be non-negative")
        if self.phenotype_model not in ("rules", "network"):
            raise ValueError("phenotype_model must be 'rules' or 'network'")
        if self.inhibition_threshold < 1:
            raise ValueError("inhibition_threshold must be at least 1")
        if self.death_threshold < 0.0 or self.hypoxia_threshold < self.death_threshold:
            raise ValueError("need 0 <= death_threshold <= hypoxia_threshold")
        if self.glucose_death_threshold < 0.0 or self.glucose_threshold < self.glucose_death_threshold:
            raise ValueError("need 0 <= glucose_death_threshold <= glucose_threshold")
        if self.placement_factor <= 0.0:
            raise ValueError("placement_factor must be positive")

    @property
    def uses_network(self) -> bool:
        return self.phenotype_model == "network"

    @classmethod
    def oxygen_dependent(cls, **overrides) -> LifecycleParams:
        """Defaults with the illustrative oxygen thresholds switched on."""
        values = {"hypoxia_threshold": 8.0, "death_threshold": 2.0, "anoxic_death_rate": 0.5}
        values.update(overrides)
        return cls(**values)

    def native(self, dt: float) -> _lib.LifecycleParamsC:
        return _lib.LifecycleParamsC(
            dt=dt,
            death_rate=self.death_rate,
            anoxic_death_rate=self.anoxic_death_rate,
            division_rate=self.division_rate,
            inhibition_threshold=min(int(self.inhibition_threshold), 2**31 - 1),
            hypoxia_threshold=self.hypoxia_threshold,
            death_threshold=self.death_threshold,
            glucose_threshold=self.glucose_threshold,
            glucose_death_threshold=self.glucose_death_threshold,
            necrosis_requires_glucose=1 if self.necrosis_requires_glucose else 0,
            phenotype_model=1 if self.uses_network else 0,
            apoptosis_rate=self.apoptosis_rate,
            necrosis_rate=self.necrosis_rate,
        )


def decide_lifecycle(population, params: LifecycleParams, dt: float) -> None:
    """Every living cell's decisions for one step of ``dt`` [h]: death, state, and whether it
    divides (``divide_flag``). No host synchronisation; nothing is created until
    :func:`commit_divisions` runs."""
    if dt <= 0.0:
        raise ValueError("dt must be positive")
    n = population.count
    if n == 0:
        return
    p = population
    with profiling.stage("decide"):
        _decide(p, params, dt, n)


def _decide(p, params: LifecycleParams, dt: float, n: int) -> None:
    _lib.call(
        "wbc_lifecycle_decide",
        ctypes.byref(params.native(dt)),
        n,
        _lib.ptr(p.cell_state),
        _lib.ptr(p.age),
        _lib.ptr(p.neighbor_count),
        _lib.ptr(p.oxygen_local),
        _lib.ptr(p.glucose_local),
        _lib.ptr(p.fate_flags),
        _lib.ptr(p.rng_state),
        _lib.ptr(p.divide_flag),
        _lib.stream(p.device),
    )


def scan_divisions(population) -> None:
    """Inclusive prefix sum of ``divide_flag[:count]`` into ``division_offset`` and the daughter
    total into the population's device counter (no host sync)."""
    n = population.count
    workspace, total = population.scan_workspace()
    with profiling.stage("scan", launches=3):
        _scan(population, n, workspace, total)


def _scan(population, n, workspace, total) -> None:
    _lib.call(
        "wbc_division_scan",
        n,
        _lib.ptr(population.divide_flag),
        _lib.ptr(population.division_offset),
        _lib.ptr(total),
        _lib.ptr(workspace),
        workspace.numel() * 4,
        _lib.stream(population.device),
    )


def place_daughters(population, params: LifecycleParams) -> None:
    """Launch the placement over the current prefix (after :func:`scan_divisions`)."""
    with profiling.stage("place"):
        _place(population, params)


def _place(p, params: LifecycleParams) -> None:
    _lib.call(
        "wbc_place_daughters",
        p.count,
        float(params.placement_factor),
        _lib.ptr(p.divide_flag),
        _lib.ptr(p.division_offset),
        _lib.ptr(p.position),
        _lib.ptr(p.radius),
        _lib.ptr(p.cell_state),
        _lib.ptr(p.cell_type),
        _lib.ptr(p.age),
        _lib.ptr(p.oxygen_local),
        _lib.ptr(p.glucose_local),
        _lib.ptr(p.rng_state),
        _lib.ptr(p.velocity),
        _lib.ptr(p.neighbor_count),
        _lib.ptr(p.fate_flags),
        _lib.stream(p.device),
    )


def commit_divisions(population, params: LifecycleParams) -> int:
    """Append the daughters of the cells whose ``divide_flag`` is set; returns their number.

    One host-device synchronisation (reading that number). Raises :class:`CapacityError`,
    leaving no daughter placed, if the population would exceed its capacity; the decisions
    already taken (deaths, state changes, consumed draws) are kept.
    """
    n = population.count
    if n == 0:
        return 0
    scan_divisions(population)
    _, total = population.scan_workspace()
    n_daughters = int(total.item())  # the single sync
    if n_daughters == 0:
        return 0
    if n + n_daughters > population.capacity:
        raise CapacityError(
            f"{n_daughters} divisions would bring the population to {n + n_daughters} cells, "
            f"above the allocated capacity of {population.capacity}"
        )
    place_daughters(population, params)
    population.count = n + n_daughters
    return n_daughters


def lifecycle_step(population, params: LifecycleParams, dt: float) -> int:
    """:func:`decide_lifecycle` then :func:`commit_divisions`; returns the daughters created."""
    decide_lifecycle(population, params, dt)
    return commit_divisions(population, params)

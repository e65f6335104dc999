"""Many independent spheroids advanced together (a parameter sweep on one GPU).

Each member is an ordinary plain-run setup: a ``CellPopulation``, its ``NeighborGrid``, its
``OxygenField`` and its ``LifecycleParams`` / ``ContactParams``. ``SpheroidBatch.step`` advances
all of them by one cell step with one launch per stage for the whole batch (the per-cell stages
over a work list of 256-cell chunks, the field solves as one persistent launch over the tiles of
every grid), in the order of :func:`simulation.simulator.cell_step`: deposit + conversion, field
solve, sampling, lifecycle (decisions, prefix sum, daughters), then the contact substeps. Every
member's results are bit-identical to running ``cell_step`` on it alone.

Cell counts stay on the device during the steps (``counts``), so nothing synchronises with the
host and a step can be captured in a CUDA graph (:meth:`SpheroidBatch.capture`).
:meth:`SpheroidBatch.sync` copies the counts back into the populations. A member whose daughters
would exceed its capacity places none and reports ``WBC_ERR_CAPACITY`` in ``status`` instead of
raising ``CapacityError``.

The reference has no batched form; its sweep runs one experiment after another
(simulation/sweep.py:132-139).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.cells.lifecycle import LifecycleParams
from warpbiocell_gb300.cells.mechanics import ContactParams
from warpbiocell_gb300.fields import diffusion
from warpbiocell_gb300.fields.diffusion import SolveReport, sor_params
from warpbiocell_gb300.simulation.simulator import TimeStepping


@dataclass
class BatchMember:
    population: object  # CellPopulation
    grid: object  # NeighborGrid
    oxygen: object  # OxygenField
    lifecycle: LifecycleParams
    contact: ContactParams


class SpheroidBatch:
    def __init__(self, members: list[BatchMember], stepping: TimeStepping):
        if not members:
            raise ValueError("a batch needs at least one member")
        self.members = list(members)
        self.stepping = stepping
        self.device = members[0].population.device
        settings = members[0].oxygen.settings
        for m in members:
            if m.population.device != self.device:
                raise RuntimeError("every member must live on the same device")
            if m.oxygen.settings != settings:
                raise ValueError("every member must use the same solver settings")
            if m.oxygen.species.produces:
                raise ValueError("batched members have a single consumed species (oxygen)")
            m.contact.check_substep(stepping.dt_mechanics)
        self.settings = settings
        n = len(members)
        self.counts = torch.tensor([m.population.count for m in members], dtype=torch.int32, device=self.device)
        self.status = torch.zeros(n, dtype=torch.int32, device=self.device)
        self._graph = None
        self.launches_per_step = 0

        insts = (_lib.BatchInstanceC * n)()
        for k, m in enumerate(members):
            insts[k] = self._instance(m)
        self._insts = insts
        plan_bytes = int(_lib.load().wbc_batch_plan_bytes(n, insts))
        if plan_bytes == 0:
            raise ValueError("batch too large")
        self._plan = torch.empty(plan_bytes, dtype=torch.uint8, device=self.device)
        self.native = _lib.BatchC()
        _lib.call("wbc_batch_prepare", n, insts, _lib.ptr(self._plan), plan_bytes, ctypes.byref(self.native),
                  _lib.stream(self.device))

        items = (_lib.SorBatchItemC * n)()
        for k, m in enumerate(members):
            fld = m.oxygen
            params = sor_params(fld.field, fld.species.kinetics, settings.omega, False, 1.0)
            ws = diffusion._workspace(fld.field, params)
            items[k] = _lib.SorBatchItemC(params, _lib.ptr(fld.field.fixed_or_none()), _lib.ptr(fld.density), None,
                                          None, _lib.ptr(fld.field.values), _lib.ptr(ws))
        self._items = items
        sor_bytes = int(_lib.load().wbc_sor_batch_plan_bytes(n))
        self._sor_plan = torch.empty(sor_bytes, dtype=torch.uint8, device=self.device)
        self.sor = _lib.SorBatchC()
        self._prepare_solver(None)

    def _prepare_solver(self, weights) -> None:
        n = len(self.members)
        w = (ctypes.c_float * n)(*weights) if weights is not None else None
        _lib.call("wbc_sor_batch_prepare", n, self._items, w, int(self.settings.check_every),
                  int(self.settings.max_sweeps), float(self.settings.tolerance), _lib.ptr(self._sor_plan),
                  self._sor_plan.numel(), ctypes.byref(self.sor), _lib.stream(self.device))

    def rebalance(self, sweeps=None) -> None:
        """Re-plan the batched solve for each member's expected sweep count: ``sweeps`` (one
        number per member, e.g. the mean of recent solves) or else the last solve's count. The
        planner groups members of similar sweep counts into waves and gives each the tiles that
        make a wave's members end together. Drops a captured graph; call :meth:`capture` again."""
        if sweeps is None:
            sweeps = [r.sweeps for r in self.reports()]
        sweeps = [float(x) for x in sweeps]
        if len(sweeps) != len(self.members):
            raise ValueError(f"need {len(self.members)} sweep counts, got {len(sweeps)}")
        weights = [float(m.oxygen.geometry.node_count) * max(1.0, x) for m, x in zip(self.members, sweeps)]
        self._prepare_solver(weights)
        self._graph = None

    def _instance(self, m: BatchMember) -> _lib.BatchInstanceC:
        pop, grid, fld = m.population, m.grid, m.oxygen
        grid.reserve(pop.capacity)
        dens = fld.densities
        w = fld.species.uptake_weights
        inst = _lib.BatchInstanceC()
        inst.capacity = pop.capacity
        for name in ("position", "radius", "cell_state", "cell_type", "age", "oxygen_local", "glucose_local",
                     "rng_state", "velocity", "neighbor_count", "divide_flag", "division_offset", "fate_flags"):
            setattr(inst, name, _lib.ptr(getattr(pop, name)))
        inst.grid = grid.struct
        inst.query_radius = float(m.contact.query_radius)
        inst.contact_rate = float(m.contact.rate)
        inst.contact_dt = float(self.stepping.dt_mechanics)
        inst.contact_substeps = self.stepping.mechanics_substeps
        inst.geom = fld.geometry.native()
        # the batched deposit writes into the member's own 32-bit accumulator and produces only the
        # combined uptake density; the member's per-state densities are converted from the same sums
        # when they are read, as on the plain path
        inst.accumulator = _lib.ptr(dens.accumulator_for_writing())
        inst.density = None
        inst.uptake_density = _lib.ptr(fld.density)
        inst.uptake_weights = (ctypes.c_float * 4)(*[float(x) for x in w])
        inst.inv_voxel_volume = 1.0 / fld.geometry.voxel_volume
        inst.field = _lib.ptr(fld.field.values)
        inst.lifecycle = m.lifecycle.native(self.stepping.dt_cells)
        inst.placement_factor = float(m.lifecycle.placement_factor)
        return inst

    # ---- stepping ----------------------------------------------------------------------------------
    def _launch_step(self) -> None:
        b, st = ctypes.byref(self.native), _lib.stream(self.device)
        counts = _lib.ptr(self.counts)
        _lib.call("wbc_batch_deposit", b, counts, st)
        _lib.call("wbc_sor_batch_solve", ctypes.byref(self.sor), st)
        _lib.call("wbc_batch_sample", b, counts, st)
        _lib.call("wbc_batch_lifecycle", b, counts, _lib.ptr(self.status), st)
        for _ in range(self.stepping.mechanics_substeps):
            _lib.call("wbc_batch_grid_build", b, counts, st)
            _lib.call("wbc_batch_contact", b, counts, st)

    def step(self, steps: int = 1) -> None:
        """Advance every member by ``steps`` cell steps (replaying the captured graph if any)."""
        for _ in range(steps):
            if self._graph is not None:
                self._graph.replay()
            else:
                self._launch_step()

    def capture(self) -> None:
        """Record one step as a CUDA graph; later :meth:`step` calls replay it."""
        graph = torch.cuda.CUDAGraph()
        before = _lib.launch_count()
        stream = torch.cuda.Stream(device=self.device)
        stream.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(stream):
            with torch.cuda.graph(graph, stream=stream):
                self._launch_step()
        torch.cuda.current_stream(self.device).wait_stream(stream)
        self._graph = graph
        self.launches_per_step = _lib.launch_count() - before  # kernels in one replay

    # ---- host view ---------------------------------------------------------------------------------
    def sync(self) -> list[int]:
        """Copy the device cell counts into the populations; returns them."""
        counts = self.counts.cpu().tolist()
        for m, c in zip(self.members, counts):
            m.population.count = int(c)
        return counts

    def status_codes(self) -> list[int]:
        return self.status.cpu().tolist()

    def reports(self) -> list[SolveReport]:
        """The last field solve of every member."""
        n = len(self.members)
        reps = (_lib.SorReportC * n)()
        _lib.call("wbc_sor_batch_reports", ctypes.byref(self.sor), reps, _lib.stream(self.device))
        return [SolveReport(sweeps=int(r.sweeps), residual=float(r.residual), converged=bool(r.converged))
                for r in reps]

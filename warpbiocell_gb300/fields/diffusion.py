"""Reaction-diffusion solvers on a ScalarField with Michaelis-Menten uptake
(reference: fields/diffusion.py:18-154).

``solve_steady_state`` is the production path: red-black SOR sweeps in place from the field's
current values (warm start), ``check_every`` sweeps per native call (``wbc_sor_sweeps``, which
also reduces the max-norm residual on the device), one host read of the residual per check,
exactly the reference's cadence and stopping rule. ``explicit_step`` (FTCS) is for validation.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from warpbiocell_gb300 import _lib, profiling
from warpbiocell_gb300.fields.scalar_field import ScalarField


@dataclass(frozen=True)
class UptakeKinetics:
    """``q(O) = uptake_max * O / (michaelis_k + O)`` per consuming cell; ``diffusion`` D [um^2/h]."""

    diffusion: float
    uptake_max: float
    michaelis_k: float

    def __post_init__(self):
        if self.diffusion <= 0.0:
            raise ValueError("diffusion coefficient must be positive")
        if self.uptake_max < 0.0 or self.michaelis_k <= 0.0:
            raise ValueError("uptake_max must be non-negative and michaelis_k positive")


@dataclass(frozen=True)
class SolverSettings:
    """Red-black SOR settings: relaxation ``omega`` in (0, 2), a hard ``max_sweeps`` budget, the
    dimensionless max-norm residual ``tolerance`` and ``check_every`` sweeps between residual
    checks (each check is one host sync). In float32 the residual bottoms out near
    1e-7 * omega / (2 - omega), so tolerances below ~1e-6 may never be met."""

    omega: float = 1.5
    max_sweeps: int = 2000
    tolerance: float = 1.0e-5
    check_every: int = 20

    def __post_init__(self):
        if not 0.0 < self.omega < 2.0:
            raise ValueError("omega must lie in (0, 2)")
        if self.max_sweeps < 1 or self.check_every < 1:
            raise ValueError("max_sweeps and check_every must be positive")
        if self.tolerance <= 0.0:
            raise ValueError("tolerance must be positive")


@dataclass(frozen=True)
class SolveReport:
    sweeps: int
    residual: float
    converged: bool


def _source_args(field: ScalarField, production, source, source_k):
    prod = production if production is not None else None
    has_source = 1 if source is not None else 0
    return prod, has_source, source, float(source_k)


def sor_params(field: ScalarField, kinetics: UptakeKinetics, omega: float, has_source: int = 0,
               source_k: float = 1.0) -> _lib.SorParamsC:
    """Kernel parameters, each rounded to float32 from the same double expression the reference uses."""
    geom = field.geometry
    nx, ny, nz = geom.shape
    bc_x, bc_y, bc_z = field.boundary_flags
    reference = field.boundary_value if field.boundary_value > 0.0 else 1.0
    return _lib.SorParamsC(nx=nx, ny=ny, nz=nz, bc_x=bc_x, bc_y=bc_y, bc_z=bc_z, omega=omega,
                           dx2_over_D=geom.dx**2 / kinetics.diffusion, uptake_max=kinetics.uptake_max,
                           michaelis_k=kinetics.michaelis_k, reference=reference, has_source=has_source,
                           source_k=source_k)


def sor_chunk(field: ScalarField, density: torch.Tensor, params: _lib.SorParamsC, sweeps: int,
              residual_buffer: torch.Tensor | None, production=None, source=None) -> None:
    """``sweeps`` red-black sweeps (and the residual into ``residual_buffer[0]`` when given)."""
    with profiling.stage("sor", launches=2 * int(sweeps) + (1 if residual_buffer is not None else 0)):
        _lib.call("wbc_sor_sweeps", ctypes.byref(params), int(sweeps), _lib.ptr(field.fixed_or_none()),
                  _lib.ptr(density), _lib.ptr(production), _lib.ptr(source), _lib.ptr(field.values),
                  _lib.ptr(residual_buffer), _lib.stream(field.device))


class PendingSolve:
    """A solve launched without waiting for its report (``solve_steady_state(..., defer=True)``):
    the report is copied into a pinned host record in stream order and read by :meth:`result`,
    which waits only if the stream has not passed the solve yet (in a cell step it has: the
    division count is read after the solve)."""

    def __init__(self, field: ScalarField, record: torch.Tensor, on_result=None):
        self._field = field
        self._record = record
        self._event = torch.cuda.Event()
        self._event.record(torch.cuda.current_stream(field.device))
        self._on_result = on_result
        self._report: SolveReport | None = None

    def result(self) -> SolveReport:
        if self._report is None:
            self._event.synchronize()
            rep = _lib.SorReportC()
            _lib.call("wbc_sor_report_decode", self._record.data_ptr(), ctypes.byref(rep))  # pinned host memory
            last_solve.update(sweeps=rep.sweeps, path=rep.path, tiles=rep.tiles, strips=rep.strips)
            self._report = SolveReport(sweeps=int(rep.sweeps), residual=float(rep.residual),
                                       converged=bool(rep.converged))
            if getattr(self._field, "_pending_solve", None) is self:
                self._field._pending_solve = None
            if self._on_result is not None:
                self._on_result(self._report)
        return self._report


def _report_record(field: ScalarField) -> torch.Tensor:
    """The field's pinned host record for deferred reports (allocated once, 128-byte aligned)."""
    record = getattr(field, "_report_record", None)
    if record is None:
        nbytes = int(_lib.load().wbc_sor_report_record_bytes())
        raw = torch.empty(nbytes + 128, dtype=torch.uint8, pin_memory=True)
        off = (-raw.data_ptr()) % 128
        record = raw[off:off + nbytes]
        field._report_record = record
    return record


def solve_steady_state(
    field: ScalarField,
    density: torch.Tensor,
    kinetics: UptakeKinetics,
    settings: SolverSettings,
    residual_buffer: torch.Tensor,
    production: torch.Tensor | None = None,
    source: torch.Tensor | None = None,
    source_k: float = 1.0,
    defer: bool = False,
    on_result=None,
):
    """Iterate SOR sweeps in place, starting from the field's current values (warm start).

    ``production`` [conc/h] is an optional zero-order source per node, scaled by
    ``S/(source_k + S)`` of the ``source`` field when one is given. With ``defer`` the solve is
    launched without waiting for its report and a :class:`PendingSolve` is returned (its
    ``result()`` gives the SolveReport and calls ``on_result`` with it).
    """
    if residual_buffer.dtype != torch.float32 or residual_buffer.device != field.device or residual_buffer.numel() < 1:
        raise ValueError("residual_buffer must be a float32 tensor of at least one element on the field's device")
    prod, has_source, src, source_k = _source_args(field, production, source, source_k)
    params = sor_params(field, kinetics, settings.omega, has_source, source_k)
    workspace = _workspace(field, params)
    report = _lib.SorReportC()
    if solver_tuning is not None:
        tuning = _lib.SorTuningC(*solver_tuning)
    elif solver_path != 1:
        tuning = _autotuned(field, params, settings, density, prod, src, workspace)
    else:
        tuning = None
    # The library writes the final residual into residual_buffer[0] itself (no extra kernel).
    if defer:
        earlier = getattr(field, "_pending_solve", None)
        if earlier is not None:
            earlier.result()  # its record is about to be reused
        record = _report_record(field)
        with profiling.stage("sor"):
            _lib.call("wbc_sor_solve_deferred", ctypes.byref(params), int(settings.check_every),
                      int(settings.max_sweeps), float(settings.tolerance), _lib.ptr(field.fixed_or_none()),
                      _lib.ptr(density), _lib.ptr(prod), _lib.ptr(src), _lib.ptr(field.values),
                      _lib.ptr(residual_buffer), record.data_ptr(), _lib.ptr(workspace), workspace.numel(),
                      int(solver_path), ctypes.byref(tuning) if tuning is not None else None,
                      _lib.stream(field.device))
        pending = PendingSolve(field, record, on_result)
        field._pending_solve = pending
        return pending
    with profiling.stage("sor"):
        _lib.call("wbc_sor_solve", ctypes.byref(params), int(settings.check_every), int(settings.max_sweeps),
                  float(settings.tolerance), _lib.ptr(field.fixed_or_none()), _lib.ptr(density), _lib.ptr(prod),
                  _lib.ptr(src), _lib.ptr(field.values), _lib.ptr(residual_buffer), ctypes.byref(report),
                  _lib.ptr(workspace), workspace.numel(), int(solver_path),
                  ctypes.byref(tuning) if tuning is not None else None, _lib.stream(field.device))
    last_solve.update(sweeps=report.sweeps, path=report.path, tiles=report.tiles, strips=report.strips)
    result = SolveReport(sweeps=int(report.sweeps), residual=float(report.residual), converged=bool(report.converged))
    if on_result is not None:
        on_result(result)
    return result


# 0: the shared-memory resident solver when the grid fits on chip, else streaming colour launches;
# 1: streaming colour launches only; 2: resident only (an error if the grid does not fit).
solver_path = 0
# (tiles, strips) for the resident solver: None = measured by the autotuner on the
# first solve of each grid configuration; zeros = the library's built-in choice.
solver_tuning: tuple[int, int] | None = None
# sweeps / path / CTA count of the most recent solve (for benchmarks and tests)
last_solve: dict = {}
# autotuner results: key -> (tiles, strips, us_per_sweep)
autotune_cache: dict = {}


def _autotuned(field: ScalarField, params: _lib.SorParamsC, settings: SolverSettings, density: torch.Tensor,
               prod, src, workspace: torch.Tensor) -> _lib.SorTuningC:
    """The resident solver's tuning for this grid configuration, timed once by ``wbc_sor_autotune``
    on a copy of the field and cached (every tuning gives the same field bits)."""
    fixed = field.fixed_or_none()
    key = (str(field.device), field.geometry.shape, (params.bc_x, params.bc_y, params.bc_z), prod is not None,
           bool(params.has_source), fixed is not None, int(settings.check_every))
    hit = autotune_cache.get(key)
    if hit is None:
        best = _lib.SorTuningC()
        us = ctypes.c_float(0.0)
        scratch = torch.empty_like(field.values)
        _lib.call("wbc_sor_autotune", ctypes.byref(params), int(settings.check_every), _lib.ptr(fixed),
                  _lib.ptr(density), _lib.ptr(prod), _lib.ptr(src), _lib.ptr(field.values), _lib.ptr(scratch),
                  _lib.ptr(workspace), workspace.numel(), ctypes.byref(best), ctypes.byref(us),
                  _lib.stream(field.device))
        hit = (int(best.tiles), int(best.strips), float(us.value))
        autotune_cache[key] = hit
    return _lib.SorTuningC(*hit[:2])


def _workspace(field: ScalarField, params: _lib.SorParamsC) -> torch.Tensor:
    """Scratch of the solver (control block, halo exchange and coefficient planes), per field."""
    nbytes = int(_lib.load().wbc_sor_solve_workspace_bytes(ctypes.byref(params)))
    ws = getattr(field, "_sor_workspace", None)
    if ws is None or ws.numel() < nbytes:
        ws = torch.empty(nbytes, dtype=torch.uint8, device=field.device)
        object.__setattr__(field, "_sor_workspace", ws)
    return ws


def max_stable_dt(field: ScalarField, kinetics: UptakeKinetics) -> float:
    """Explicit-scheme stability limit ``dx^2 / (6 D)`` [h]."""
    return field.geometry.dx**2 / (6.0 * kinetics.diffusion)


def explicit_step(
    field: ScalarField,
    density: torch.Tensor,
    kinetics: UptakeKinetics,
    dt: float,
    scratch: torch.Tensor,
    production: torch.Tensor | None = None,
    source: torch.Tensor | None = None,
    source_k: float = 1.0,
) -> None:
    """One FTCS step into ``scratch``, copied back so ``field.values`` stays the same tensor."""
    limit = max_stable_dt(field, kinetics)
    if dt > limit * (1.0 + 1.0e-6):
        raise ValueError(f"dt = {dt:.3g} h exceeds the explicit stability limit dx^2/(6D) = {limit:.3g} h")
    prod, has_source, src, source_k = _source_args(field, production, source, source_k)
    geom = field.geometry
    nx, ny, nz = geom.shape
    bc_x, bc_y, bc_z = field.boundary_flags
    params = _lib.SorParamsC(nx=nx, ny=ny, nz=nz, bc_x=bc_x, bc_y=bc_y, bc_z=bc_z, omega=1.0,
                             dx2_over_D=kinetics.diffusion / geom.dx**2, uptake_max=kinetics.uptake_max,
                             michaelis_k=kinetics.michaelis_k, reference=1.0, has_source=has_source,
                             source_k=source_k)
    _lib.call("wbc_ftcs_step", ctypes.byref(params), float(dt), _lib.ptr(field.fixed), _lib.ptr(density),
              _lib.ptr(prod), _lib.ptr(src), _lib.ptr(field.values), _lib.ptr(scratch), _lib.stream(field.device))
    field.values.copy_(scratch)

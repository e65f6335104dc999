"""Differentiable coupled steady state with a hand-written adjoint (torch.autograd.Function).

Forward model, from fixed initial positions and radii:

    K contact steps      x_{t+1} = x_t + dt v(x_t; rate = stiffness / damping)   (contact_substep)
    uptake deposit       U = per-cell uptake capacities Vmax_i spread with trilinear weights
    steady O2 field      sum_nb u - (6 + h U / (Km + u)) u = 0, Dirichlet faces at O_b, h = dx^2 / D

``CoupledSteadyState.apply(vmax, km, diffusion, boundary, stiffness, model)`` returns the field
``u`` (flat, one value per node) and the final positions ``x_K``; any torch loss of them can be
differentiated with respect to the per-cell ``vmax`` and the scalars ``km``, ``diffusion``,
``boundary`` and ``stiffness``. The backward pass solves the transposed linearised field operator
with red-black SOR, forms the parameter and position gradients, and runs the contact steps in
reverse over the neighbour sets of the forward steps, recomputing the positions of each
segment of sqrt(K) steps from a checkpoint (so memory grows with sqrt(K) position arrays and
sqrt(K) hash grids). The K forward steps run in one launch; each segment takes one launch to
recompute and one to reverse. The steady field is the fp32 SOR solution corrected by Newton steps
whose residuals are formed in FP64, and the field adjoint is refined the same way, so the
gradients match an FP64 evaluation of the model.

The reference has no differentiable path; the forward pieces are its contact law, deposit and SOR
update (kernels/mechanics_kernels.py:26-67, kernels/field_kernels.py:78-116 and 185-212) with a
per-cell uptake capacity in place of the per-state one.
"""

from __future__ import annotations

import ctypes
import math

import torch

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.cells.mechanics import ContactParams
from warpbiocell_gb300.fields.diffusion import SolverSettings, UptakeKinetics, solve_steady_state, sor_params
from warpbiocell_gb300.fields.scalar_field import GridGeometry, ScalarField
from warpbiocell_gb300.spatial.neighbors import NeighborGrid


class AdjointSpheroid:
    """The model's fixed data (initial cells, grid, step count) and its device buffers."""

    def __init__(self, positions: torch.Tensor, radii: torch.Tensor, geometry: GridGeometry, steps: int, dt: float,
                 contact: ContactParams = ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0),
                 settings: SolverSettings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=20000,
                                                           check_every=20),
                 adjoint_tolerance: float = 1e-6, device=None):
        """``adjoint_tolerance`` bounds the field adjoint's max residual relative to
        max(6 |mu|, |dL/du|)."""
        self.device = _lib.resolve_device(device if device is not None else positions.device)
        self.x0 = positions.detach().to(self.device, torch.float32).contiguous()
        self.radii = radii.detach().to(self.device, torch.float32).contiguous()
        self.n = int(self.x0.shape[0])
        if self.x0.shape != (self.n, 3) or self.radii.shape != (self.n,):
            raise ValueError("positions must be (n, 3) and radii (n,)")
        self.geometry = geometry
        self.steps = int(steps)
        if self.steps < 0:
            raise ValueError("steps must be non-negative")
        self.dt = float(dt)
        self.contact = contact
        self.settings = settings
        self.adjoint_tolerance = float(adjoint_tolerance)
        self.segment = max(1, int(math.ceil(math.sqrt(max(self.steps, 1)))))
        # Hash buckets: 64 per axis when the cells' extent (with room to move) spans fewer buckets,
        # so no two cells closer than the query radius alias; any size finds the same pairs, a
        # smaller one only scans fewer empty buckets per step.
        extent = float((self.x0.max(dim=0).values - self.x0.min(dim=0).values).max().item()) if self.n else 0.0
        dim = 64 if extent / contact.query_radius + 8 <= 64 else 128
        self.grid = NeighborGrid(contact.query_radius, dim=dim, device=self.device)
        self.grid.reserve(self.n)
        self._slots = max(2, self.segment)
        lib = _lib.load()
        ws_bytes = int(lib.wbc_contact_steps_workspace_bytes(dim, self.grid.struct.capacity, self._slots))
        self._steps_ws = torch.empty(ws_bytes + 256, dtype=torch.uint8, device=self.device)
        off = (-self._steps_ws.data_ptr()) % 256
        self._steps_ws = self._steps_ws[off:off + ws_bytes]
        nseg = max(1, (self.steps + self.segment - 1) // self.segment)
        self._checkpoints = torch.empty(nseg, self.n, 3, dtype=torch.float32, device=self.device)
        self._checkpoints_lo = torch.empty_like(self._checkpoints)
        self.velocity = torch.zeros(self.n, 3, dtype=torch.float32, device=self.device)
        self.neighbor_count = torch.zeros(self.n, dtype=torch.int32, device=self.device)
        self.accumulator = torch.zeros(geometry.node_count, dtype=torch.int64, device=self.device)
        self.uptake = torch.zeros(geometry.node_count, dtype=torch.float32, device=self.device)
        self._residual = torch.zeros(1, dtype=torch.float32, device=self.device)
        nodes = geometry.node_count
        self._diag = torch.empty(nodes, dtype=torch.float32, device=self.device)
        self._rhs = torch.empty(nodes, dtype=torch.float32, device=self.device)
        self._delta = torch.empty(nodes, dtype=torch.float32, device=self.device)
        probe = _lib.SorParamsC(nx=geometry.shape[0], ny=geometry.shape[1], nz=geometry.shape[2])
        self._workspace = torch.empty(int(_lib.load().wbc_sor_solve_workspace_bytes(ctypes.byref(probe))),
                                      dtype=torch.uint8, device=self.device)
        # Per-pass buffers (filled by the library's kernels, so a pass launches no other kernel) and
        # the field object every forward pass refills.
        self._hi = torch.empty(self.n, 3, dtype=torch.float32, device=self.device)
        self._lo = torch.empty_like(self._hi)
        self._weight = torch.empty(self.n, dtype=torch.float32, device=self.device)
        self._mean = torch.empty(257, dtype=torch.float64, device=self.device)  # WBC_MEAN_SCRATCH
        self._g = torch.empty(nodes, dtype=torch.float32, device=self.device)
        self._mu0 = torch.empty(nodes, dtype=torch.float32, device=self.device)
        self._dmu = torch.empty(nodes, dtype=torch.float32, device=self.device)
        self._phi = torch.empty(nodes, dtype=torch.float32, device=self.device)
        self._sums = torch.empty(3, dtype=torch.float64, device=self.device)
        self._rate_dot = torch.empty(1, dtype=torch.float64, device=self.device)
        self._lam_tmp = torch.empty_like(self._hi)
        self._work = torch.empty_like(self._hi)
        self._work_lo = torch.empty_like(self._hi)
        self._field_object = None
        # Newton corrections of the fp32 steady field and refinement of the adjoint solve, each to this
        # relative residual (the correction problems are solved in fp32, their residuals in FP64).
        self.newton_steps = 2
        self.refine_tolerance = 1e-6
        self.last_forward_sweeps = 0
        self.last_newton_sweeps = 0
        self.last_adjoint_sweeps = 0

    # ---- pieces ------------------------------------------------------------------------------------
    def _steps(self, pos: torch.Tensor, lo: torch.Tensor, rate: float, steps: int, checkpoints: bool = False,
               history: bool = False) -> None:
        """`steps` contact steps in place on the compensated positions pos + lo (the plain path's
        contact law, the positions kept to about 48 bits) in one launch; with `checkpoints`, x_t for
        every t % segment == 0; with `history`, the grids of the steps' starting positions are kept
        for the reverse pass and the last step only builds its grid."""
        _lib.call("wbc_contact_steps", ctypes.byref(self.grid.struct), self.n, float(self.contact.query_radius),
                  float(rate), self.dt, int(steps), _lib.ptr(pos), _lib.ptr(lo), _lib.ptr(self.radii),
                  _lib.ptr(self.velocity), _lib.ptr(self.neighbor_count),
                  _lib.ptr(self._checkpoints) if checkpoints else None,
                  _lib.ptr(self._checkpoints_lo) if checkpoints else None, self.segment, self._slots, int(history),
                  int(history), _lib.ptr(self._steps_ws), self._steps_ws.numel(), 1, _lib.stream(self.device))

    def _zero(self, t: torch.Tensor) -> None:
        _lib.call("wbc_zero", _lib.ptr(t), t.numel() * t.element_size(), _lib.stream(self.device))

    def _field(self, pos: torch.Tensor, vmax: torch.Tensor, km: float, diffusion: float, boundary: float):
        """Deposit, the fp32 steady solve, then Newton corrections with FP64 residuals: returns the
        solver parameters and the refined field (float64, flat)."""
        st = _lib.stream(self.device)
        # per-cell weights Vmax_i / mean(Vmax), the mean in FP64 by a fixed-order reduction
        _lib.call("wbc_mean", self.n, _lib.ptr(vmax), _lib.ptr(self._mean), st)
        scale = float(self._mean[0].item())
        _lib.call("wbc_divide", self.n, _lib.ptr(vmax), scale, _lib.ptr(self._weight), st)
        geom = self.geometry.native()
        _lib.call("wbc_deposit_weighted", ctypes.byref(geom), self.n, _lib.ptr(pos), _lib.ptr(self._weight),
                  _lib.ptr(self.accumulator), st)
        _lib.call("wbc_weighted_convert", self.geometry.node_count, _lib.ptr(self.accumulator),
                  scale / self.geometry.voxel_volume, _lib.ptr(self.uptake), 1, st)
        nodes = self.geometry.node_count
        if self._field_object is None:
            self._field_object = ScalarField.create(self.geometry, boundary, device=self.device)
        field = self._field_object
        field.boundary_value = float(boundary)  # a cold start from the boundary value, as a new field
        _lib.call("wbc_fill", nodes, float(boundary), _lib.ptr(field.values), st)
        kin = UptakeKinetics(diffusion, 1.0, km)
        report = solve_steady_state(field, self.uptake, kin, self.settings, self._residual)
        self.last_forward_sweeps = report.sweeps
        u64 = torch.empty(nodes, dtype=torch.float64, device=self.device)
        _lib.call("wbc_widen", nodes, _lib.ptr(field.values), _lib.ptr(u64), st)
        params = sor_params(field, kin, self.settings.omega, False, 1.0)
        sweeps = 0
        for _ in range(self.newton_steps):
            _lib.call("wbc_adjoint_newton_prepare", ctypes.byref(params), _lib.ptr(u64), _lib.ptr(self.uptake),
                      _lib.ptr(self._diag), _lib.ptr(self._rhs), st)
            self._zero(self._delta)
            sweeps += self._linear_solve(params, self._diag, self._rhs, self._delta, self.refine_tolerance)
            _lib.call("wbc_adjoint_newton_apply", nodes, _lib.ptr(self._delta), _lib.ptr(u64), st)
        self.last_newton_sweeps = sweeps
        return params, u64

    def _linear_solve(self, params, diag: torch.Tensor, rhs: torch.Tensor, x: torch.Tensor, tolerance: float) -> int:
        """diag x - sum_nb x = rhs from x's current values, in one resident launch; returns the sweeps."""
        report = _lib.SorReportC()
        ws = self._workspace
        _lib.call("wbc_sor_linear_solve", ctypes.byref(params), int(self.settings.check_every),
                  int(self.settings.max_sweeps), float(tolerance), _lib.ptr(diag), _lib.ptr(rhs), _lib.ptr(x),
                  ctypes.byref(report), _lib.ptr(ws), ws.numel(), _lib.stream(self.device))
        self.last_linear_converged = bool(report.converged)
        return int(report.sweeps)

    # ---- forward / backward ------------------------------------------------------------------------
    def forward(self, vmax: torch.Tensor, km: float, diffusion: float, boundary: float, stiffness: float):
        """(u flat, x_K); keeps the checkpoints and the field state for :meth:`backward`."""
        st = _lib.stream(self.device)
        vmax = vmax.detach()
        if vmax.dtype != torch.float32 or not vmax.is_contiguous() or vmax.device != self.device:
            vmax = vmax.to(self.device, torch.float32).contiguous()
        if vmax.shape != (self.n,):
            raise ValueError(f"vmax must have shape ({self.n},)")
        rate = float(stiffness) / self.contact.damping
        hi, lo = self._hi, self._lo
        hi.copy_(self.x0)
        self._zero(lo)
        self._steps(hi, lo, rate, self.steps, checkpoints=True)
        x64 = torch.empty(self.n, 3, dtype=torch.float64, device=self.device)
        pos = torch.empty(self.n, 3, dtype=torch.float32, device=self.device)  # positions for the deposit
        _lib.call("wbc_compensated_sum", 3 * self.n, _lib.ptr(hi), _lib.ptr(lo), _lib.ptr(x64), _lib.ptr(pos), st)
        params, u64 = self._field(pos, vmax, km, diffusion, boundary)
        uptake = torch.empty_like(self.uptake)
        uptake.copy_(self.uptake)
        self._saved = dict(pos=pos, vmax=vmax, km=float(km), diffusion=float(diffusion), boundary=float(boundary),
                           stiffness=float(stiffness), rate=rate, params=params, uptake=uptake, u64=u64)
        u = torch.empty_like(u64)
        u.copy_(u64)
        return u, x64

    def backward(self, grad_u: torch.Tensor | None, grad_x: torch.Tensor | None) -> dict:
        sv = self._saved
        st = _lib.stream(self.device)
        nodes = self.geometry.node_count
        pos, vmax, params = sv["pos"], sv["vmax"], sv["params"]
        g = self._g
        if grad_u is None:
            self._zero(g)
        else:
            self._narrow_into(grad_u, g)
        lam = torch.empty(self.n, 3, dtype=torch.float32, device=self.device)  # becomes dL/dx_0
        if grad_x is None:
            self._zero(lam)
        else:
            self._narrow_into(grad_x, lam)

        # field adjoint: (6 + h kappa) mu - sum_nb mu = dL/du at the refined field, solved in fp32 and
        # refined once with the residual in FP64 (mu = mu0 + dmu)
        u64 = sv["u64"]
        diag, rhs, mu0, dmu = self._diag, self._rhs, self._mu0, self._dmu
        _lib.call("wbc_adjoint_newton_prepare", ctypes.byref(params), _lib.ptr(u64), _lib.ptr(sv["uptake"]),
                  _lib.ptr(diag), _lib.ptr(rhs), st)
        self._zero(mu0)
        self._zero(dmu)
        sweeps = self._linear_solve(params, diag, g, mu0, self.adjoint_tolerance)
        converged = self.last_linear_converged
        _lib.call("wbc_adjoint_linear_residual", ctypes.byref(params), _lib.ptr(diag), _lib.ptr(g), _lib.ptr(mu0),
                  _lib.ptr(rhs), st)
        sweeps += self._linear_solve(params, diag, rhs, dmu, self.adjoint_tolerance)
        phi, sums = self._phi, self._sums
        _lib.call("wbc_adjoint_field_grads", ctypes.byref(params), _lib.ptr(u64), _lib.ptr(sv["uptake"]),
                  _lib.ptr(mu0), _lib.ptr(dmu), _lib.ptr(diag), _lib.ptr(g), _lib.ptr(phi), _lib.ptr(sums), st)
        self.last_adjoint_converged = converged and self.last_linear_converged
        self.last_adjoint_sweeps = sweeps
        h = params.dx2_over_D
        grad_vmax = torch.empty(self.n, dtype=torch.float32, device=self.device)
        coef = -h / self.geometry.voxel_volume
        geom = self.geometry.native()
        _lib.call("wbc_adjoint_cells", ctypes.byref(geom), self.n, _lib.ptr(pos), _lib.ptr(vmax), _lib.ptr(phi),
                  coef, _lib.ptr(grad_vmax), _lib.ptr(lam), st)

        # mechanics in reverse, one checkpointed segment at a time: the segment's positions are
        # recomputed from its checkpoint in one launch that keeps each step's grid, then its steps
        # run in reverse in one launch over those grids
        rate = sv["rate"]
        rate_dot, lam_tmp, work, work_lo = self._rate_dot, self._lam_tmp, self._work, self._work_lo
        self._zero(rate_dot)
        for seg in range((self.steps + self.segment - 1) // self.segment - 1, -1, -1):
            start = seg * self.segment
            stop = min(self.steps, start + self.segment)
            work.copy_(self._checkpoints[seg])
            work_lo.copy_(self._checkpoints_lo[seg])
            self._steps(work, work_lo, rate, stop - start, history=True)
            _lib.call("wbc_adjoint_steps", ctypes.byref(self.grid.struct), self.n, float(self.contact.query_radius),
                      float(rate), self.dt, stop - start, 1, _lib.ptr(lam), _lib.ptr(lam_tmp), _lib.ptr(rate_dot),
                      self._slots, _lib.ptr(self._steps_ws), self._steps_ws.numel(), 1, st)
        d_km, d_diffusion_times_d, d_boundary = sums.tolist()
        d_rate = self.dt * float(rate_dot.item())
        return dict(vmax=grad_vmax, km=d_km, diffusion=d_diffusion_times_d / sv["diffusion"], boundary=d_boundary,
                    stiffness=d_rate / self.contact.damping, x0=lam)

    def _narrow_into(self, src: torch.Tensor, dst: torch.Tensor) -> None:
        """dst = src as float32 (a float64 gradient narrowed by the library, a float32 one copied)."""
        src = src.detach().reshape(dst.shape)
        if src.dtype == torch.float64 and src.is_contiguous() and src.device == self.device:
            _lib.call("wbc_narrow", dst.numel(), _lib.ptr(src), _lib.ptr(dst), _lib.stream(self.device))
        else:
            dst.copy_(src)


class CoupledSteadyState(torch.autograd.Function):
    """``u, x_K = CoupledSteadyState.apply(vmax, km, diffusion, boundary, stiffness, model)``."""

    @staticmethod
    def forward(ctx, vmax, km, diffusion, boundary, stiffness, model: AdjointSpheroid):
        # NVTX ranges name the passes for profilers (the backward runs on autograd's device thread)
        torch.cuda.nvtx.range_push("wbc_adjoint_forward")
        try:
            u, x = model.forward(vmax.detach(), float(km), float(diffusion), float(boundary), float(stiffness))
        finally:
            torch.cuda.nvtx.range_pop()
        ctx.model = model
        ctx.scalar_like = [torch.as_tensor(v) for v in (km, diffusion, boundary, stiffness)]
        return u, x

    @staticmethod
    def backward(ctx, grad_u, grad_x):
        torch.cuda.nvtx.range_push("wbc_adjoint_backward")
        try:
            grads = ctx.model.backward(grad_u, grad_x)
        finally:
            torch.cuda.nvtx.range_pop()
        like = ctx.scalar_like

        def scalar(value, ref):
            return torch.tensor(value, dtype=ref.dtype if ref.is_floating_point() else torch.float64,
                                device=ref.device)

        return (grads["vmax"], scalar(grads["km"], like[0]), scalar(grads["diffusion"], like[1]),
                scalar(grads["boundary"], like[2]), scalar(grads["stiffness"], like[3]), None)

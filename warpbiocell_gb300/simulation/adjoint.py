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
segment of sqrt(K) steps from a checkpoint (so memory grows with sqrt(K) position arrays).

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
        self.grid = NeighborGrid(contact.query_radius, dim=128, device=self.device)
        self.grid.reserve(self.n)
        self.velocity = torch.zeros(self.n, 3, dtype=torch.float32, device=self.device)
        self.neighbor_count = torch.zeros(self.n, dtype=torch.int32, device=self.device)
        self.accumulator = torch.zeros(geometry.node_count, dtype=torch.int64, device=self.device)
        self.uptake = torch.zeros(geometry.node_count, dtype=torch.float32, device=self.device)
        self._residual = torch.zeros(1, dtype=torch.float32, device=self.device)
        self.last_forward_sweeps = 0
        self.last_adjoint_sweeps = 0

    # ---- pieces ------------------------------------------------------------------------------------
    def _step(self, pos: torch.Tensor, rate: float) -> None:
        """One contact step in place (the plain path's contact_substep)."""
        st = _lib.stream(self.device)
        _lib.call("wbc_grid_build", ctypes.byref(self.grid.struct), self.n, _lib.ptr(pos), _lib.ptr(self.radii), st)
        _lib.call("wbc_contact_substep", ctypes.byref(self.grid.struct), self.n, float(self.contact.query_radius),
                  float(rate), self.dt, _lib.ptr(pos), _lib.ptr(self.velocity), _lib.ptr(self.neighbor_count), st)

    def _field(self, pos: torch.Tensor, vmax: torch.Tensor, km: float, diffusion: float, boundary: float):
        st = _lib.stream(self.device)
        scale = float(vmax.mean().item())
        weight = (vmax / scale).to(torch.float32).contiguous()
        geom = self.geometry.native()
        _lib.call("wbc_deposit_weighted", ctypes.byref(geom), self.n, _lib.ptr(pos), _lib.ptr(weight),
                  _lib.ptr(self.accumulator), st)
        _lib.call("wbc_weighted_convert", self.geometry.node_count, _lib.ptr(self.accumulator),
                  scale / self.geometry.voxel_volume, _lib.ptr(self.uptake), 1, st)
        field = ScalarField.create(self.geometry, boundary, device=self.device)
        kin = UptakeKinetics(diffusion, 1.0, km)
        report = solve_steady_state(field, self.uptake, kin, self.settings, self._residual)
        self.last_forward_sweeps = report.sweeps
        return field, report

    # ---- forward / backward ------------------------------------------------------------------------
    def forward(self, vmax: torch.Tensor, km: float, diffusion: float, boundary: float, stiffness: float):
        """(u flat, x_K); keeps the checkpoints and the field state for :meth:`backward`."""
        rate = float(stiffness) / self.contact.damping
        pos = self.x0.clone()
        self._checkpoints = []
        for t in range(self.steps):
            if t % self.segment == 0:
                self._checkpoints.append(pos.clone())
            self._step(pos, rate)
        field, report = self._field(pos, vmax, km, diffusion, boundary)
        self._saved = dict(pos=pos, vmax=vmax.detach().contiguous(), km=float(km), diffusion=float(diffusion),
                           boundary=float(boundary), stiffness=float(stiffness), rate=rate, field=field,
                           uptake=self.uptake.clone())
        return field.values.reshape(-1).clone(), pos.clone()

    def backward(self, grad_u: torch.Tensor | None, grad_x: torch.Tensor | None) -> dict:
        sv = self._saved
        st = _lib.stream(self.device)
        nodes = self.geometry.node_count
        pos, vmax, field = sv["pos"], sv["vmax"], sv["field"]
        g = torch.zeros(nodes, dtype=torch.float32, device=self.device) if grad_u is None else \
            grad_u.detach().to(torch.float32).reshape(-1).contiguous()
        lam = torch.zeros(self.n, 3, dtype=torch.float32, device=self.device) if grad_x is None else \
            grad_x.detach().to(torch.float32).contiguous().clone()

        # field adjoint
        kin = UptakeKinetics(sv["diffusion"], 1.0, sv["km"])
        params = sor_params(field, kin, self.settings.omega, False, 1.0)
        mu = torch.zeros(nodes, dtype=torch.float32, device=self.device)
        kappa = torch.empty_like(mu)
        phi = torch.empty_like(mu)
        sums = torch.zeros(3, dtype=torch.float64, device=self.device)
        bits = torch.zeros(2, dtype=torch.int32, device=self.device)
        report = _lib.SorReportC()
        _lib.call("wbc_adjoint_field_solve", ctypes.byref(params), _lib.ptr(field.values), _lib.ptr(sv["uptake"]),
                  _lib.ptr(g), _lib.ptr(mu), _lib.ptr(kappa), int(self.settings.check_every),
                  int(self.settings.max_sweeps), self.adjoint_tolerance, _lib.ptr(phi), _lib.ptr(sums),
                  _lib.ptr(bits), ctypes.byref(report), st)
        self.last_adjoint_converged = bool(report.converged)
        self.last_adjoint_sweeps = int(report.sweeps)
        d_km, d_diffusion_times_d, d_boundary = sums.tolist()
        h = params.dx2_over_D
        grad_vmax = torch.empty(self.n, dtype=torch.float32, device=self.device)
        coef = -h / self.geometry.voxel_volume
        geom = self.geometry.native()
        _lib.call("wbc_adjoint_cells", ctypes.byref(geom), self.n, _lib.ptr(pos), _lib.ptr(vmax), _lib.ptr(phi),
                  coef, _lib.ptr(grad_vmax), _lib.ptr(lam), st)

        # mechanics in reverse, one checkpointed segment at a time
        rate = sv["rate"]
        d_rate = torch.zeros((), dtype=torch.float64, device=self.device)
        lam_next = torch.empty_like(lam)
        vdot = torch.empty(self.n, dtype=torch.float32, device=self.device)
        for seg in range(len(self._checkpoints) - 1, -1, -1):
            start = seg * self.segment
            stop = min(self.steps, start + self.segment)
            states = [self._checkpoints[seg].clone()]
            for _ in range(start, stop - 1):
                nxt = states[-1].clone()
                self._step(nxt, rate)
                states.append(nxt)
            for t in range(stop - 1, start - 1, -1):
                xt = states[t - start]
                _lib.call("wbc_grid_build", ctypes.byref(self.grid.struct), self.n, _lib.ptr(xt),
                          _lib.ptr(self.radii), st)
                _lib.call("wbc_adjoint_contact", ctypes.byref(self.grid.struct), self.n,
                          float(self.contact.query_radius), float(rate), self.dt, _lib.ptr(lam), _lib.ptr(lam_next),
                          _lib.ptr(vdot), st)
                d_rate += vdot.sum(dtype=torch.float64)
                lam, lam_next = lam_next, lam
        d_rate = self.dt * float(d_rate.item())
        return dict(vmax=grad_vmax, km=d_km, diffusion=d_diffusion_times_d / sv["diffusion"], boundary=d_boundary,
                    stiffness=d_rate / self.contact.damping, x0=lam)


class CoupledSteadyState(torch.autograd.Function):
    """``u, x_K = CoupledSteadyState.apply(vmax, km, diffusion, boundary, stiffness, model)``."""

    @staticmethod
    def forward(ctx, vmax, km, diffusion, boundary, stiffness, model: AdjointSpheroid):
        u, x = model.forward(vmax.detach(), float(km), float(diffusion), float(boundary), float(stiffness))
        ctx.model = model
        ctx.scalar_like = [torch.as_tensor(v) for v in (km, diffusion, boundary, stiffness)]
        return u, x

    @staticmethod
    def backward(ctx, grad_u, grad_x):
        grads = ctx.model.backward(grad_u, grad_x)
        like = ctx.scalar_like

        def scalar(value, ref):
            return torch.tensor(value, dtype=ref.dtype if ref.is_floating_point() else torch.float64,
                                device=ref.device)

        return (grads["vmax"], scalar(grads["km"], like[0]), scalar(grads["diffusion"], like[1]),
                scalar(grads["boundary"], like[2]), scalar(grads["stiffness"], like[3]), None)

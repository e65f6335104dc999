"""The hand-written adjoint of the coupled steady state (K contact steps, per-cell uptake deposit,
steady Michaelis-Menten field) against central finite differences of an FP64 re-run of the same
model (the oracle's double-precision contact steps, exact deposit weights and a double SOR solve
to 1e-13), for a loss of the field and of the cells' distances from their centroid."""

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from warpbiocell_gb300.cells.initialization import clipped_normal_radii, uniform_ball
from warpbiocell_gb300.cells.mechanics import ContactParams
from warpbiocell_gb300.fields.scalar_field import GridGeometry
from warpbiocell_gb300.simulation.adjoint import AdjointSpheroid, CoupledSteadyState

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
VMAX = 20e-18 / 1.3e-21 * 3600.0


def _problem(n=1200, ball=100.0, nodes=25, dx=10.0, steps=9, seed=5):
    pos = uniform_ball(n, ball, seed=seed)
    radii = clipped_normal_radii(n, seed=seed + 1)
    half = 0.5 * (nodes - 1) * dx
    geom = GridGeometry(origin=(-half, -half, -half), dx=dx, shape=(nodes,) * 3)
    contact = ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0)
    model = AdjointSpheroid(torch.from_numpy(pos), torch.from_numpy(radii), geom, steps, 0.1, contact=contact,
                            adjoint_tolerance=1e-6, device=DEV)
    rng = np.random.default_rng(seed + 2)
    vmax = (VMAX * np.exp(0.3 * rng.standard_normal(n))).astype(np.float32)
    theta = dict(km=1.0, diffusion=7.2e6, boundary=60.0, stiffness=1.0)
    return model, pos, radii, geom, vmax, theta, rng


def _radii_from_centroid(x):
    return (x - x.mean(axis=0)).norm(dim=1) if isinstance(x, torch.Tensor) else \
        np.linalg.norm(x - x.mean(axis=0), axis=1)


def test_adjoint_gradients_match_fp64_central_differences():
    model, pos, radii, geom, vmax, theta, rng = _problem()
    # targets: the model at parameters perturbed by up to +-20%
    pert = {k: v * (1.0 + 0.2 * (2 * rng.random() - 1)) for k, v in theta.items()}
    vmax_t = torch.from_numpy(vmax * (1.0 + 0.2 * (2 * rng.random(vmax.size) - 1)).astype(np.float32)).to(DEV)
    with torch.no_grad():
        u_t, x_t = model.forward(vmax_t, pert["km"], pert["diffusion"], pert["boundary"], pert["stiffness"])
    u_t64, rho_t64 = u_t.double().cpu().numpy(), _radii_from_centroid(x_t.double()).cpu().numpy()

    v = torch.from_numpy(vmax).to(DEV).requires_grad_(True)
    scal = {k: torch.tensor(val, dtype=torch.float64, requires_grad=True) for k, val in theta.items()}
    u, x = CoupledSteadyState.apply(v, scal["km"], scal["diffusion"], scal["boundary"], scal["stiffness"], model)
    rho_t = torch.from_numpy(rho_t64).to(DEV)
    loss = ((u.double() - u_t.double()) ** 2).sum() + ((_radii_from_centroid(x.double()) - rho_t) ** 2).sum()
    loss.backward()
    assert model.last_adjoint_sweeps > 0

    def loss64(vm, km, diffusion, boundary, stiffness):
        field, p, _ = orc.adjoint_forward_f64(pos, radii, vm, orc.Geometry(geom.origin, geom.dx, geom.shape),
                                              model.steps, model.dt, stiffness / model.contact.damping,
                                              model.contact.query_radius, model.contact.query_radius, 128,
                                              diffusion, km, boundary)
        return float(((field - u_t64) ** 2).sum() + ((_radii_from_centroid(p) - rho_t64) ** 2).sum())

    vm64 = vmax.astype(np.float64)
    base = dict(theta)
    rel = 1e-4
    errors = {}
    for name in ("km", "diffusion", "boundary", "stiffness"):
        h = rel * base[name]
        hi, lo = dict(base), dict(base)
        hi[name] += h
        lo[name] -= h
        fd = (loss64(vm64, **hi) - loss64(vm64, **lo)) / (2 * h)
        got = float(scal[name].grad)
        errors[name] = abs(got - fd) / abs(fd)
    for k in range(2):
        d = np.where(rng.random(vmax.size) < 0.5, -1.0, 1.0)
        fd = (loss64(vm64 * (1 + rel * d), **base) - loss64(vm64 * (1 - rel * d), **base)) / (2 * rel)
        got = float((v.grad.double().cpu().numpy() * vm64 * d).sum())
        errors[f"vmax_dir{k}"] = abs(got - fd) / abs(fd)
    print("relative errors vs FP64 central differences:", {k: f"{e:.2e}" for k, e in errors.items()})
    assert max(errors.values()) < 1e-4, errors

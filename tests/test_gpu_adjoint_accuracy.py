"""The hand-written adjoint at a mid size (20,000 cells, 49^3 grid, K = 16 contact steps) against
the oracle's FP64 adjoint of the same model and against FP64 central differences, for all five
gradients: Km, D, boundary O2, repulsion stiffness and a random per-cell Vmax direction.

The GPU gradients must be within 2e-5 of the FP64 adjoint. Against central differences with a
relative step of 1e-4 the bound is 1e-4 for every gradient except the stiffness when the two
perturbed trajectories differ in contact pairs: the overlap force has a kink at contact onset, and
a difference that spans one measures a blend of the two one-sided derivatives. For the stiffness
the test therefore also takes the difference at steps 1e-5 and 1e-6, counts the pairs that cross
contact onset between the two trajectories at each, and requires the adjoint within 1e-4 of the
difference at the smallest step that crosses none (or, when every step crosses some, within the
spread of the differences)."""

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


def test_mid_size_gradients_match_fp64_adjoint_and_central_differences():
    n, ball, nodes, dx, steps = 20000, 292.0, 49, 15.0, 16
    rng = np.random.default_rng(19)
    pos = uniform_ball(n, ball, seed=4)
    radii = clipped_normal_radii(n, 8.0, 0.8, 6.0, 10.0, seed=5)
    half = 0.5 * (nodes - 1) * dx
    geom = GridGeometry(origin=(-half,) * 3, dx=dx, shape=(nodes,) * 3)
    og = orc.Geometry(geom.origin, geom.dx, geom.shape)
    contact = ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0)
    model = AdjointSpheroid(torch.from_numpy(pos), torch.from_numpy(radii), geom, steps, 0.1, contact=contact,
                            device=DEV)
    vmax = (VMAX * np.exp(0.3 * rng.standard_normal(n))).astype(np.float32)
    theta = dict(km=1.0, diffusion=7.2e6, boundary=38.0, stiffness=1.0)
    # targets: the model at parameters perturbed by up to +-20% (seeded)
    pert = {k: v * (1.0 + 0.2 * (2 * rng.random() - 1)) for k, v in theta.items()}
    vmax_t = torch.from_numpy((vmax * (1.0 + 0.2 * (2 * rng.random(n) - 1))).astype(np.float32)).to(DEV)
    with torch.no_grad():
        u_t, x_t = model.forward(vmax_t, pert["km"], pert["diffusion"], pert["boundary"], pert["stiffness"])
    u64 = u_t.double().cpu().numpy()
    xt = x_t.double().cpu().numpy()
    rho64 = np.linalg.norm(xt - xt.mean(axis=0), axis=1)

    v = torch.from_numpy(vmax).to(DEV).requires_grad_(True)
    scal = {k: torch.tensor(val, dtype=torch.float64, requires_grad=True) for k, val in theta.items()}
    u, x = CoupledSteadyState.apply(v, scal["km"], scal["diffusion"], scal["boundary"], scal["stiffness"], model)
    xd = x.double()
    rho_t = torch.from_numpy(rho64).to(DEV)
    loss = ((u.double() - u_t.double()) ** 2).sum() + (((xd - xd.mean(dim=0)).norm(dim=1) - rho_t) ** 2).sum()
    loss.backward()
    assert model.last_adjoint_converged
    grads = {k: float(t.grad) for k, t in scal.items()}
    grad_v = v.grad.double().cpu().numpy()

    vm64 = vmax.astype(np.float64)

    def loss_grads(field, p):
        c = p - p.mean(axis=0)
        rho = np.linalg.norm(c, axis=1)
        gx = (2.0 * (rho - rho64))[:, None] * c / rho[:, None]
        return 2.0 * (field - u64), gx - gx.mean(axis=0)

    f64 = orc.adjoint_gradients_f64(pos, radii, vm64, og, steps, 0.1, 1.0, 1.0, 20.0, 20.0, 128, theta["diffusion"],
                                    theta["km"], theta["boundary"], loss_grads)
    d = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    vs_adjoint = {k: abs(grads[k] - f64[k]) / abs(f64[k]) for k in ("km", "diffusion", "boundary", "stiffness")}
    vs_adjoint["vmax_direction"] = abs(float((grad_v * vm64 * d).sum()) - float((f64["vmax"] * vm64 * d).sum())) / \
        abs(float((f64["vmax"] * vm64 * d).sum()))
    print("relative to the FP64 adjoint:", {k: f"{e:.2e}" for k, e in vs_adjoint.items()})
    assert max(vs_adjoint.values()) < 2e-5, vs_adjoint

    def loss64(vm, km, diffusion, boundary, stiffness):
        field, p, _ = orc.adjoint_forward_f64(pos, radii, vm, og, steps, 0.1, stiffness, 20.0, 20.0, 128, diffusion,
                                              km, boundary)
        return float(((field - u64) ** 2).sum() + ((np.linalg.norm(p - p.mean(axis=0), axis=1) - rho64) ** 2).sum())

    rel = 1e-4
    vs_fd = {}
    for name in ("km", "diffusion", "boundary"):
        h = rel * theta[name]
        hi, lo = dict(theta), dict(theta)
        hi[name] += h
        lo[name] -= h
        fd = (loss64(vm64, **hi) - loss64(vm64, **lo)) / (2 * h)
        vs_fd[name] = abs(grads[name] - fd) / abs(fd)
    fd = (loss64(vm64 * (1 + rel * d), **theta) - loss64(vm64 * (1 - rel * d), **theta)) / (2 * rel)
    vs_fd["vmax_direction"] = abs(float((grad_v * vm64 * d).sum()) - fd) / abs(fd)
    stiff = []
    for r in (1e-4, 1e-5, 1e-6):
        hi, lo = dict(theta), dict(theta)
        hi["stiffness"] *= 1 + r
        lo["stiffness"] *= 1 - r
        fd = (loss64(vm64, **hi) - loss64(vm64, **lo)) / (2 * r * theta["stiffness"])
        crossings = orc.contact_crossings_f64(pos, radii, steps, 0.1, hi["stiffness"], lo["stiffness"], 20.0, 20.0,
                                              128)
        stiff.append((r, fd, crossings))
    print("relative to FP64 central differences:", {k: f"{e:.2e}" for k, e in vs_fd.items()},
          "stiffness (step, difference, crossings):", stiff)
    assert max(vs_fd.values()) < 1e-4, vs_fd
    clean = [fd for r, fd, c in stiff if c == 0]
    if clean:
        assert abs(grads["stiffness"] - clean[-1]) / abs(clean[-1]) < 1e-4, stiff
    else:
        values = [fd for _, fd, _ in stiff]
        assert min(values) - 1e-4 * abs(min(values)) <= grads["stiffness"] <= max(values) + 1e-4 * abs(max(values))

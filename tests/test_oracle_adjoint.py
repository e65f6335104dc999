"""The oracle's FP64 adjoint of the coupled steady state (the reference for the GPU adjoint's
gradients) against central finite differences of the oracle's FP64 forward, on the CPU: every
gradient (Km, D, boundary O2, stiffness and a random per-cell Vmax direction) within 1e-6, and the
count of contact-onset crossings a finite difference in the stiffness steps over."""

import numpy as np

from oracle import oracle as orc
from warpbiocell_gb300.cells.initialization import clipped_normal_radii, uniform_ball

VMAX = 20e-18 / 1.3e-21 * 3600.0


def _model(n=1200, ball=100.0, nodes=25, dx=10.0, steps=9):
    pos = uniform_ball(n, ball, seed=5).astype(np.float64)
    radii = clipped_normal_radii(n, seed=6).astype(np.float64)
    half = 0.5 * (nodes - 1) * dx
    geom = orc.Geometry((-half,) * 3, dx, (nodes,) * 3)
    vmax = VMAX * np.exp(0.3 * np.random.default_rng(7).standard_normal(n))
    return pos, radii, geom, vmax, steps


def test_fp64_adjoint_matches_fp64_central_differences():
    pos, radii, geom, vmax, steps = _model()
    theta = dict(km=1.0, diffusion=7.2e6, boundary=60.0, stiffness=1.0)

    def forward(vm, km, diffusion, boundary, stiffness):
        return orc.adjoint_forward_f64(pos, radii, vm, geom, steps, 0.1, stiffness, 20.0, 20.0, 128, diffusion, km,
                                       boundary)[:2]

    u_t, x_t = forward(vmax * 1.1, 1.15, 7.2e6 * 0.9, 55.0, 1.12)
    rho_t = np.linalg.norm(x_t - x_t.mean(axis=0), axis=1)

    def loss(vm, **th):
        u, x = forward(vm, **th)
        return ((u - u_t) ** 2).sum() + ((np.linalg.norm(x - x.mean(axis=0), axis=1) - rho_t) ** 2).sum()

    def loss_grads(u, x):
        c = x - x.mean(axis=0)
        rho = np.linalg.norm(c, axis=1)
        gx = (2.0 * (rho - rho_t))[:, None] * c / rho[:, None]
        return 2.0 * (u - u_t), gx - gx.mean(axis=0)

    g = orc.adjoint_gradients_f64(pos, radii, vmax, geom, steps, 0.1, 1.0, 1.0, 20.0, 20.0, 128, 7.2e6, 1.0, 60.0,
                                  loss_grads)
    rel = 1e-4
    for name in ("km", "diffusion", "boundary", "stiffness"):
        h = rel * theta[name]
        hi, lo = dict(theta), dict(theta)
        hi[name] += h
        lo[name] -= h
        fd = (loss(vmax, **hi) - loss(vmax, **lo)) / (2 * h)
        assert abs(g[name] - fd) <= 1e-6 * abs(fd), (name, g[name], fd)
    d = np.where(np.random.default_rng(8).random(vmax.size) < 0.5, -1.0, 1.0)
    fd = (loss(vmax * (1 + rel * d), **theta) - loss(vmax * (1 - rel * d), **theta)) / (2 * rel)
    got = float((g["vmax"] * vmax * d).sum())
    assert abs(got - fd) <= 1e-6 * abs(fd), (got, fd)
    # at this step no contact pair starts or ends between the two trajectories
    assert orc.contact_crossings_f64(pos, radii, steps, 0.1, 1.0 + rel, 1.0 - rel, 20.0, 20.0, 128) == 0


def test_contact_crossings_counts_pairs_that_touch_in_one_trajectory_only():
    # two cells 15 um apart with radii 7.4 and 7.5: not touching at rest; a third cell pushes the
    # second towards the first only when the push is strong enough
    pos = np.array([[0.0, 0.0, 0.0], [15.0, 0.0, 0.0], [24.0, 0.0, 0.0]])
    radii = np.array([7.4, 7.5, 9.0])
    assert orc.contact_crossings_f64(pos, radii, 3, 0.1, 1.0, 1.0, 20.0, 20.0, 128) == 0
    assert orc.contact_crossings_f64(pos, radii, 3, 0.1, 0.01, 1.0, 20.0, 20.0, 128) > 0

"""The fused contact steps (many binning + contact substeps in one cooperative launch) and their
fused reverse, against the separate launches they replace: positions, velocities, neighbour
counts, checkpoints and the kept grids bit for bit, the reverse's adjoint positions bit for bit
and its rate derivative to summation order."""

import ctypes

import numpy as np
import pytest
import torch

from warpbiocell_gb300 import _lib
from warpbiocell_gb300.cells.initialization import clipped_normal_radii, uniform_ball
from warpbiocell_gb300.spatial.neighbors import NeighborGrid

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _setup(n, ball, dim, seed=3):
    pos = torch.as_tensor(uniform_ball(n, ball, seed=seed), device=DEV)
    radii = torch.as_tensor(clipped_normal_radii(n, seed=seed + 1), device=DEV)
    grid = NeighborGrid(20.0, dim=dim, device=DEV)
    grid.reserve(n)
    return pos, radii, grid


def _workspace(grid, slots):
    nbytes = int(_lib.load().wbc_contact_steps_workspace_bytes(grid.dim, grid.struct.capacity, slots))
    raw = torch.empty(nbytes + 256, dtype=torch.uint8, device=DEV)
    off = (-raw.data_ptr()) % 256
    return raw[off:off + nbytes]


def _separate_steps(pos, radii, grid, steps, rate, dt):
    n = pos.shape[0]
    vel = torch.zeros_like(pos)
    nc = torch.zeros(n, dtype=torch.int32, device=DEV)
    st = _lib.stream(torch.device(DEV))
    history = []
    for _ in range(steps):
        _lib.call("wbc_grid_build", ctypes.byref(grid.struct), n, _lib.ptr(pos), _lib.ptr(radii), st)
        history.append((grid.bucket_start.clone(), grid.bucket_count.clone(), grid.sorted_id[:n].clone(),
                        grid.sorted_xyzr[:n].clone()))
        _lib.call("wbc_contact_substep", ctypes.byref(grid.struct), n, 20.0, rate, dt, _lib.ptr(pos), _lib.ptr(vel),
                  _lib.ptr(nc), st)
    return vel, nc, history


@pytest.mark.parametrize("n, ball, dim, steps, every", [(3000, 90.0, 128, 9, 3), (20000, 170.0, 64, 7, 4),
                                                        (1, 10.0, 16, 3, 1)])
def test_fused_steps_bitwise_equal_separate_launches(n, ball, dim, steps, every):
    pos, radii, grid = _setup(n, ball, dim)
    ref = pos.clone()
    vel_ref, nc_ref, _ = _separate_steps(ref, radii, grid, steps, 1.0, 0.1)
    got = pos.clone()
    vel = torch.zeros_like(got)
    nc = torch.zeros(n, dtype=torch.int32, device=DEV)
    cps = torch.full(((steps + every - 1) // every, n, 3), -1.0, device=DEV)
    ws = _workspace(grid, 2)
    _lib.call("wbc_contact_steps", ctypes.byref(grid.struct), n, 20.0, 1.0, 0.1, steps, _lib.ptr(got), None,
              _lib.ptr(radii), _lib.ptr(vel), _lib.ptr(nc), _lib.ptr(cps), None, every, 2, 0, 0, _lib.ptr(ws),
              ws.numel(), 1, _lib.stream(torch.device(DEV)))
    torch.cuda.synchronize()
    assert torch.equal(got, ref) and torch.equal(vel, vel_ref) and torch.equal(nc, nc_ref)
    # checkpoints: x_t before step t for t = 0, every, 2 every, ...
    replay = pos.clone()
    for k in range(cps.shape[0]):
        assert torch.equal(cps[k], replay)
        _separate_steps(replay, radii, grid, min(every, steps - k * every), 1.0, 0.1)


def test_fused_history_grids_and_reverse_match_separate_launches():
    """The reverse over the grids the fused steps kept equals the separate reverse kernel over the
    separate launches' grids (so the kept grids are those grids)."""
    n, steps, rate, dt = 5000, 6, 1.3, 0.1
    pos, radii, grid = _setup(n, 110.0, 64)
    x0 = pos.clone()
    _, _, history = _separate_steps(x0.clone(), radii, grid, steps, rate, dt)
    ws = _workspace(grid, steps)
    work = x0.clone()
    vel = torch.zeros_like(work)
    nc = torch.zeros(n, dtype=torch.int32, device=DEV)
    st = _lib.stream(torch.device(DEV))
    _lib.call("wbc_contact_steps", ctypes.byref(grid.struct), n, 20.0, rate, dt, steps, _lib.ptr(work), None,
              _lib.ptr(radii), _lib.ptr(vel), _lib.ptr(nc), None, None, 1, steps, 1, 1, _lib.ptr(ws), ws.numel(), 1, st)
    # the positions after steps - 1 steps (the last step only builds its grid)
    ref = x0.clone()
    _separate_steps(ref, radii, grid, steps - 1, rate, dt)
    assert torch.equal(work, ref)
    lam0 = torch.as_tensor(np.random.default_rng(1).standard_normal((n, 3)).astype(np.float32), device=DEV)
    # reverse through the separate kernel, over the separate launches' grids
    lam = lam0.clone()
    lam_next = torch.empty_like(lam)
    vdot = torch.empty(n, dtype=torch.float32, device=DEV)
    total = 0.0
    for t in range(steps - 1, -1, -1):
        start, count, ids, xyzr = history[t]
        grid.bucket_start.copy_(start)
        grid.bucket_count.copy_(count)
        grid.sorted_id[:n].copy_(ids)
        grid.sorted_xyzr[:n].copy_(xyzr)
        _lib.call("wbc_adjoint_contact", ctypes.byref(grid.struct), n, 20.0, rate, dt, _lib.ptr(lam),
                  _lib.ptr(lam_next), _lib.ptr(vdot), st)
        total += float(vdot.double().sum())
        lam, lam_next = lam_next, lam
    got = lam0.clone()
    tmp = torch.empty_like(got)
    rate_dot = torch.zeros(1, dtype=torch.float64, device=DEV)
    _lib.call("wbc_adjoint_steps", ctypes.byref(grid.struct), n, 20.0, rate, dt, steps, 0, _lib.ptr(got),
              _lib.ptr(tmp), _lib.ptr(rate_dot), steps, _lib.ptr(ws), ws.numel(), 1, st)
    torch.cuda.synchronize()
    assert torch.equal(got, lam)
    assert abs(float(rate_dot.item()) - total) <= 1e-9 * abs(total)


def test_compensated_steps_track_fp64():
    """Compensated positions (float + low part) follow the oracle's FP64 contact steps several times
    more closely than plain float positions, which round at every step; what remains is the float
    force evaluation (the overlap r_i + r_j - d loses digits to cancellation)."""
    from oracle import oracle as orc

    n, steps = 4000, 16
    pos, radii, grid = _setup(n, 100.0, 64, seed=9)
    x64 = pos.double().cpu().numpy().copy()
    r64 = radii.double().cpu().numpy()
    vel64 = np.zeros_like(x64)
    nc64 = np.zeros(n, dtype=np.int32)
    for _ in range(steps):
        orc.lib().orc_contact_substep_f64(orc.c_int32(n), orc.P(x64), orc.P(r64), orc.f32(20.0), orc.c_int32(128),
                                          orc.c_double(20.0), orc.c_double(1.0), orc.c_double(0.1), orc.P(vel64),
                                          orc.P(nc64))
    ws = _workspace(grid, 2)
    st = _lib.stream(torch.device(DEV))
    vel = torch.zeros_like(pos)
    nc = torch.zeros(n, dtype=torch.int32, device=DEV)
    hi = pos.clone()
    lo = torch.zeros_like(pos)
    _lib.call("wbc_contact_steps", ctypes.byref(grid.struct), n, 20.0, 1.0, 0.1, steps, _lib.ptr(hi), _lib.ptr(lo),
              _lib.ptr(radii), _lib.ptr(vel), _lib.ptr(nc), None, None, 1, 2, 0, 0, _lib.ptr(ws), ws.numel(), 1, st)
    plain = pos.clone()
    _lib.call("wbc_contact_steps", ctypes.byref(grid.struct), n, 20.0, 1.0, 0.1, steps, _lib.ptr(plain), None,
              _lib.ptr(radii), _lib.ptr(vel), _lib.ptr(nc), None, None, 1, 2, 0, 0, _lib.ptr(ws), ws.numel(), 1, st)
    torch.cuda.synchronize()
    comp_err = np.abs(hi.double().cpu().numpy() + lo.double().cpu().numpy() - x64).max()
    plain_err = np.abs(plain.double().cpu().numpy() - x64).max()
    ulp = float(np.spacing(np.float32(100.0)))
    assert torch.equal(nc.cpu(), torch.as_tensor(nc64))
    print("max position error against FP64 (um): compensated", comp_err, "plain float", plain_err, "ulp", ulp)
    assert comp_err < 2.0 * ulp, (comp_err, plain_err)
    assert plain_err > 3.0 * comp_err, (comp_err, plain_err)

"""Failure detection of the solver's device waits, without a GPU fault: the grid barrier of the
resident SOR solver, run by wbc_sor_wait_selftest with CTAs that never arrive (a flag nothing
sets), gives up after its bounded polls and reports WBC_ERR_TIMEOUT; the context stays usable and
the next solve is bit-identical to the oracle's."""

import time

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from warpbiocell_gb300 import _lib
from warpbiocell_gb300.fields.diffusion import SolverSettings
from warpbiocell_gb300.fields.oxygen import OxygenField, OxygenParams
from warpbiocell_gb300.fields.scalar_field import GridGeometry

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _selftest(ctas, missing, rounds):
    lib = _lib.load()
    ws = torch.zeros(1 << 16, dtype=torch.uint8, device=DEV)  # control block + barrier flags
    return lib.wbc_sor_wait_selftest(ctas, missing, rounds, _lib.ptr(ws), ws.numel(), _lib.stream(torch.device(DEV)))


def test_barrier_completes_when_every_cta_arrives():
    assert _selftest(16, 0, 200) == _lib.WBC_OK
    assert _selftest(1, 0, 5) == _lib.WBC_OK


def test_barrier_times_out_when_a_cta_never_arrives_and_the_context_survives():
    start = time.perf_counter()
    rc = _selftest(8, 1, 1)
    elapsed = time.perf_counter() - start
    assert rc == _lib.WBC_ERR_TIMEOUT
    assert "timed out" in _lib.last_error()
    assert elapsed < 60.0
    assert _selftest(8, 0, 10) == _lib.WBC_OK  # the same context runs barriers again
    # ... and a solve, bit for bit as the oracle's
    geom = GridGeometry.centered_cube(240.0, 20.0)
    settings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=4000, check_every=10)
    ox = OxygenField(geom, OxygenParams(boundary_value=30.0), settings, device=DEV)
    x, y, z = np.meshgrid(*geom.node_coordinates(), indexing="ij")
    density = np.where(x**2 + y**2 + z**2 < 80.0**2, 2.4e-4, 0.0).astype(np.float32)
    ox.density.copy_(torch.as_tensor(density, device=DEV))
    report = ox.solve_steady_state()
    assert report.converged
    values = np.full(geom.shape, np.float32(30.0))
    kin = ox.species.kinetics
    params = orc.sor_params(orc.Geometry(geom.origin, geom.dx, geom.shape), ox.field.boundary_flags,
                            ox.field.boundary_value, kin.diffusion, kin.uptake_max, kin.michaelis_k, 1.8, 0, 1.0)
    sweeps, _, ok = orc.solve_steady_state(params, settings, np.zeros(geom.shape, np.int32), density, values)
    assert (report.sweeps, ok) == (sweeps, True)
    np.testing.assert_array_equal(ox.numpy(), values)

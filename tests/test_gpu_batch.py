"""Batched spheroids against plain runs: every member of a SpheroidBatch must end bit-identical to
running cell_step on it alone (populations, fields, deposits and densities, cell counts, solver
sweeps), with and without CUDA-graph capture of the step."""

import numpy as np
import pytest
import torch

from warpbiocell_gb300.cells.initialization import clipped_normal_radii, uniform_ball
from warpbiocell_gb300.cells.lifecycle import LifecycleParams
from warpbiocell_gb300.cells.mechanics import ContactParams, make_neighbor_grid
from warpbiocell_gb300.cells.state import CellPopulation
from warpbiocell_gb300.fields.diffusion import SolverSettings
from warpbiocell_gb300.fields.oxygen import OxygenField, OxygenParams
from warpbiocell_gb300.fields.scalar_field import GridGeometry
from warpbiocell_gb300.simulation.batch import BatchMember, SpheroidBatch
from warpbiocell_gb300.simulation.simulator import TimeStepping, cell_step

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
SETTINGS = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=400, check_every=20)
STEPPING = TimeStepping(dt_cells=0.1, dt_mechanics=0.1)
CONTACT = ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0, wall_rate=4.0)
# (cells, ball radius, grid nodes per side, spacing, boundary O2, seed)
SPECS = [(600, 90.0, 21, 12.0, 20.0, 1), (1500, 130.0, 25, 14.0, 38.0, 2), (3200, 170.0, 31, 14.0, 100.0, 3),
         (900, 110.0, 23, 12.5, 60.0, 4)]


def _member(cells, ball, nodes, dx, boundary, seed, lifecycle):
    pos = uniform_ball(cells, ball, seed=seed)
    radii = clipped_normal_radii(cells, seed=seed + 100)
    pop = CellPopulation.from_numpy(pos, radii, capacity=2 * cells, device=DEV, seed=seed)
    geom = GridGeometry.centered_cube(dx * (nodes - 1), dx)
    oxygen = OxygenField(geom, OxygenParams(diffusion_coefficient=7.2e6, uptake_max=5.54e7, michaelis_k=1.0,
                                            boundary_value=boundary), SETTINGS, device=DEV)
    return BatchMember(pop, make_neighbor_grid(CONTACT, DEV), oxygen, lifecycle, CONTACT)


def _lifecycle():
    return LifecycleParams(division_rate=0.8, death_rate=0.02, anoxic_death_rate=0.5, inhibition_threshold=14,
                           hypoxia_threshold=5.0, death_threshold=1.0)


def _snapshot(m):
    pop = m.population
    n = pop.count
    arrays = [pop.position[:n], pop.radius[:n], pop.cell_state[:n], pop.age[:n], pop.oxygen_local[:n],
              pop.rng_state, pop.velocity[:n], pop.neighbor_count[:n]]
    # the field, the solver's uptake density, and the per-state densities converted on reading
    # from the last deposit's sums
    fields = [m.oxygen.field.values, m.oxygen.density, m.oxygen.densities.density, m.oxygen.densities.accumulator]
    return n, [a.cpu().numpy().copy() for a in arrays + fields]


def _plain(steps):
    out = []
    for spec in SPECS:
        m = _member(*spec, _lifecycle())
        sweeps = []
        for _ in range(steps):
            rep = cell_step(m.population, m.grid, m.lifecycle, m.contact, STEPPING, oxygen=m.oxygen)
            sweeps.append(rep.field_sweeps)
        out.append((_snapshot(m), sweeps))
    return out


@pytest.mark.parametrize("graph", [False, True])
def test_batch_members_bitwise_equal_plain_runs(graph):
    steps = 5
    plain = _plain(steps)
    members = [_member(*spec, _lifecycle()) for spec in SPECS]
    batch = SpheroidBatch(members, STEPPING)
    if graph:
        batch.step(1)  # the first steps outside the graph (warm up the autotuned paths)
        batch.step(1)
        # a plan re-made for given sweep counts (the waves and tile counts change, the bits do not)
        batch.rebalance([r.sweeps + 20 * (k % 3) for k, r in enumerate(batch.reports())])
        batch.capture()
        batch.step(steps - 2)
    else:
        for _ in range(steps):
            batch.step(1)
            reps = batch.reports()
            assert all(r.converged for r in reps)
    counts = batch.sync()
    assert batch.status_codes() == [0] * len(SPECS)
    last = batch.reports()
    for k, (m, ((n_ref, ref), sweeps)) in enumerate(zip(members, plain)):
        assert counts[k] == n_ref, k
        n, got = _snapshot(m)
        for a, b in zip(got, ref):
            np.testing.assert_array_equal(a, b, err_msg=f"member {k}")
        assert last[k].sweeps == sweeps[-1]
    assert sum(counts) > sum(spec[0] for spec in SPECS)  # divisions happened


def test_batch_capacity_overflow_sets_status():
    lifecycle = LifecycleParams(division_rate=50.0, death_rate=0.0, inhibition_threshold=1000)
    spec = SPECS[0]
    m = _member(*spec, lifecycle)
    # capacity for the initial cells only: the first divisions overflow
    pop = m.population
    small = CellPopulation.from_numpy(pop.position[: pop.count].cpu().numpy(), pop.radius[: pop.count].cpu().numpy(),
                                      capacity=pop.count, device=DEV, seed=spec[-1])
    member = BatchMember(small, make_neighbor_grid(CONTACT, DEV), m.oxygen, lifecycle, CONTACT)
    batch = SpheroidBatch([member], STEPPING)
    batch.step(1)
    assert batch.status_codes() == [-2]
    assert batch.sync() == [spec[0]]

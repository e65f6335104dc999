"""GPU parity: the CUDA path (Python drop-in API -> C-ABI -> sm_103a kernels) against the CPU
oracle on the same seeded inputs, bit for bit where the reference's algorithm is order
independent or its order is fixed (integer deposits, neighbour sets, lifecycle decisions,
slots, network states, SOR sweeps, positions), and against the reference's golden vectors and
closed forms with the reference's own tolerances. Every test is marked ``gpu``.
"""

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from warpbiocell_gb300 import _lib
from warpbiocell_gb300.cells.initialization import spherical_cluster, uniform_ball
from warpbiocell_gb300.cells.lifecycle import CapacityError, LifecycleParams, lifecycle_step
from warpbiocell_gb300.cells.mechanics import ContactParams, contact_substep, make_neighbor_grid, relax_contacts
from warpbiocell_gb300.cells.model import CellState
from warpbiocell_gb300.cells.state import CellPopulation
from warpbiocell_gb300.fields.densities import CellDensities
from warpbiocell_gb300.fields.diffusion import SolverSettings
from warpbiocell_gb300.fields.oxygen import OxygenField, OxygenParams
from warpbiocell_gb300.fields.scalar_field import Boundary, GridGeometry
from warpbiocell_gb300.metrics.population import state_counts
from warpbiocell_gb300.simulation.simulator import TimeStepping, cell_step

pytestmark = pytest.mark.gpu

DEV = "cuda:0"
R = 8.0
MIXED = (Boundary.DIRICHLET, Boundary.NEUMANN, Boundary.DIRICHLET)


def _t(a, dtype=None):
    return torch.as_tensor(np.ascontiguousarray(a), device=DEV) if dtype is None else torch.as_tensor(
        np.ascontiguousarray(a), dtype=dtype, device=DEV)


def _stream():
    return _lib.stream(torch.device(DEV))


# ---- random streams, exp ------------------------------------------------------------------------------
def test_streams_draws_and_directions_match_oracle():
    pop = CellPopulation.from_numpy(np.zeros((1000, 3), np.float32), np.full(1000, R), capacity=4096, device=DEV, seed=17)
    np.testing.assert_array_equal(pop.rng_state.cpu().numpy().view(np.uint32), orc.rng_init(17, 4096))
    state = pop.rng_state.clone()
    out = torch.zeros((4096, 8), dtype=torch.float32, device=DEV)
    _lib.call("wbc_rng_uniform", 4096, 8, _lib.ptr(state), _lib.ptr(out), _stream())
    ref_state = orc.rng_init(17, 4096)
    np.testing.assert_array_equal(out.cpu().numpy(), orc.rng_uniform(ref_state, 8))
    np.testing.assert_array_equal(state.cpu().numpy().view(np.uint32), ref_state)
    dirs = torch.zeros((4096, 3), dtype=torch.float32, device=DEV)
    _lib.call("wbc_rng_sphere", 4096, _lib.ptr(state), _lib.ptr(dirs), _stream())
    np.testing.assert_array_equal(dirs.cpu().numpy(), orc.rng_sphere(ref_state))


def test_project_exp_matches_oracle_and_cuda_expf():
    x = np.concatenate([np.linspace(-103.9, 88.7, 100001), -np.logspace(-8, 3, 10001)]).astype(np.float32)
    xt = _t(x)
    out = torch.empty_like(xt)
    _lib.call("wbc_expf_batch", x.size, _lib.ptr(xt), _lib.ptr(out), _stream())
    got = out.cpu().numpy()
    np.testing.assert_array_equal(got, orc.expf(x))
    cuda = torch.exp(xt).cpu().numpy().astype(np.float64)  # CUDA's expf (max error 2 ulp)
    normal = cuda > 1.2e-38
    ulp = np.spacing(cuda[normal].astype(np.float32)).astype(np.float64)
    assert (np.abs(got[normal] - cuda[normal]) / ulp).max() <= 3.0


# ---- deposit / density / sample -------------------------------------------------------------------------
def _pop_from(pos, states=None, capacity=None, seed=0, radii=None):
    n = pos.shape[0]
    radii = np.full(n, R, np.float32) if radii is None else radii
    return CellPopulation.from_numpy(pos, radii, capacity=capacity, device=DEV, seed=seed, states=states)


def test_deposit_bitwise_equals_oracle_and_golden(golden):
    g = golden("deposit")
    geom = GridGeometry(tuple(g["origin"]), float(g["dx"]), tuple(int(x) for x in g["shape"]))
    pop = _pop_from(g["positions"], g["states"])
    dens = CellDensities(geom, device=DEV)
    dens.deposit_fixed_point(pop)
    acc_gpu = dens.accumulator.cpu().numpy()
    ogeom = orc.Geometry(geom.origin, geom.dx, geom.shape)
    acc_ref = orc.deposit(ogeom, g["positions"], g["states"])
    np.testing.assert_array_equal(acc_gpu, acc_ref)
    dens.convert()
    d_ref, _ = orc.density_convert(ogeom, acc_ref)
    np.testing.assert_array_equal(dens.numpy(), d_ref)
    np.testing.assert_allclose(dens.numpy(), g["density"], atol=1e-8)
    # the next deposit replaces the sums (the accumulator is cleared by the deposit itself)
    dens.deposit_fixed_point(pop)
    np.testing.assert_array_equal(dens.accumulator.cpu().numpy(), acc_ref)


def test_deposit_carry_into_high_words_is_exact():
    """Crowded nodes put more than 2^32 into single words, in every way a paired 64-bit add can
    wrap: the even word of a pair (300 cells on node (2,2,2), state 0), the odd word alone (300 on
    (2,2,3)), both words in one add (600 half-way between (3,3,2) and (3,3,3), state 2), and the two
    halves of neighbouring pairs (600 half-way between (4,1,3) and (4,1,4), state 3). The sums and
    densities equal the oracle's int64 ones."""
    geom = GridGeometry((0.0, 0.0, 0.0), 10.0, (6, 6, 6))
    rng = np.random.default_rng(12)
    crowds = [((20.0, 20.0, 20.0), 300, 0), ((20.0, 20.0, 30.0), 300, 1), ((30.0, 30.0, 25.0), 600, 2),
              ((40.0, 10.0, 35.0), 600, 3)]
    pos = np.concatenate([np.tile(np.float32(at), (k, 1)) for at, k, _ in crowds] +
                         [rng.uniform(5.0, 45.0, (500, 3))]).astype(np.float32)
    states = np.concatenate([np.full(k, st) for _, k, st in crowds] + [rng.integers(0, 4, 500)]).astype(np.int32)
    crowded = sum(k for _, k, _ in crowds)
    pop = _pop_from(pos, states)
    dens = CellDensities(geom, device=DEV)
    dens.deposit_fixed_point(pop)
    ogeom = orc.Geometry(geom.origin, geom.dx, geom.shape)
    acc_ref = orc.deposit(ogeom, pos, states)
    assert (acc_ref > 2**32).sum() >= 6
    np.testing.assert_array_equal(dens.accumulator.cpu().numpy(), acc_ref)
    d_ref, _ = orc.density_convert(ogeom, acc_ref)
    np.testing.assert_array_equal(dens.numpy(), d_ref)
    # a following deposit without the crowds clears the wrap counts again
    dens.deposit_fixed_point(_pop_from(pos[crowded:], states[crowded:]))
    np.testing.assert_array_equal(dens.accumulator.cpu().numpy(), orc.deposit(ogeom, pos[crowded:], states[crowded:]))


def test_deposit_skips_cells_outside_the_grid_and_empty_populations():
    """Cells outside the trilinear support (below the origin, on or past the last node) are skipped
    as the oracle skips them, on an odd-sized grid whose z-corner pairs straddle the ends of
    columns; a deposit of no cells then leaves every sum and density zero."""
    geom = GridGeometry((-5.0, 0.0, 3.0), 7.0, (5, 6, 7))
    rng = np.random.default_rng(21)
    pos = np.concatenate([rng.uniform(-15.0, 50.0, (4000, 3)),
                          np.array([[-5.0, 0.0, 3.0], [23.0, 35.0, 45.0], [22.99, 34.99, 44.99], [-5.001, 10.0, 10.0]])]
                         ).astype(np.float32)
    states = rng.integers(0, 4, pos.shape[0]).astype(np.int32)
    ogeom = orc.Geometry(geom.origin, geom.dx, geom.shape)
    dens = CellDensities(geom, device=DEV)
    dens.deposit_fixed_point(_pop_from(pos, states))
    acc_ref = orc.deposit(ogeom, pos, states)
    assert 0 < np.count_nonzero(acc_ref) < acc_ref.size
    np.testing.assert_array_equal(dens.accumulator.cpu().numpy(), acc_ref)
    np.testing.assert_array_equal(dens.numpy(), orc.density_convert(ogeom, acc_ref)[0])
    empty = _pop_from(np.zeros((0, 3), np.float32), np.zeros(0, np.int32), capacity=16)
    dens.deposit_fixed_point(empty)
    assert not dens.accumulator.any()
    assert not dens.density.any()


def test_deposit_in_hash_grid_order_and_lazy_densities():
    """The deposit visits the cells in the order of the last binning (same sums), and the plain
    oxygen step's consuming density alone gives the per-state densities later from the same deposit."""
    pos = uniform_ball(30000, 250.0, seed=8)
    states = np.random.default_rng(8).integers(0, 4, 30000).astype(np.int32)
    geom = GridGeometry.centered_cube(600.0, 15.0)
    pop = _pop_from(pos, states)
    ogeom = orc.Geometry(geom.origin, geom.dx, geom.shape)
    acc_ref = orc.deposit(ogeom, pos, states)
    grid = make_neighbor_grid(ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0), DEV)
    grid.build(pop)
    order = pop.spatial_order()
    assert order is not None and torch.equal(order[:pop.count].sort().values.cpu(), torch.arange(pop.count).int())
    dens = CellDensities(geom, device=DEV)
    dens.deposit_fixed_point(pop)
    np.testing.assert_array_equal(dens.accumulator.cpu().numpy(), acc_ref)
    combined = torch.empty(geom.shape, dtype=torch.float32, device=DEV)
    dens.convert_combined((1.0, 1.0, 1.0, 0.0), combined)
    d_ref, c_ref = orc.density_convert(ogeom, acc_ref, (1.0, 1.0, 1.0, 0.0))
    np.testing.assert_array_equal(combined.cpu().numpy(), c_ref)
    np.testing.assert_array_equal(dens.numpy(), d_ref)


def test_deposit_large_is_order_independent_and_reproducible():
    pos = uniform_ball(200000, 600.0, seed=3)
    states = np.random.default_rng(3).integers(0, 4, 200000).astype(np.int32)
    geom = GridGeometry.centered_cube(1200.0, 15.0)
    ogeom = orc.Geometry(geom.origin, geom.dx, geom.shape)
    ref = orc.deposit(ogeom, pos, states)
    for perm_seed in (None, 1):
        p, s = pos, states
        if perm_seed is not None:
            perm = np.random.default_rng(perm_seed).permutation(len(states))
            p, s = pos[perm], states[perm]
        dens = CellDensities(geom, device=DEV)
        dens.deposit_fixed_point(_pop_from(p, s))
        np.testing.assert_array_equal(dens.accumulator.cpu().numpy(), ref)


def test_fused_convert_combine_equals_separate_passes():
    pos = uniform_ball(20000, 200.0, seed=4)
    states = np.random.default_rng(4).integers(0, 4, 20000).astype(np.int32)
    geom = GridGeometry.centered_cube(500.0, 20.0)
    ox = OxygenField(geom, OxygenParams(), device=DEV, uptake_state_factors={"hypoxic": 0.5})
    pop = _pop_from(pos, states)
    ox.deposit_uptake(pop)
    ogeom = orc.Geometry(geom.origin, geom.dx, geom.shape)
    d_ref, _ = orc.density_convert(ogeom, orc.deposit(ogeom, pos, states))
    np.testing.assert_array_equal(ox.densities.numpy(), d_ref)
    np.testing.assert_array_equal(ox.density.cpu().numpy(), orc.combine(d_ref, ox.species.uptake_weights))


def test_sample_bitwise_equals_oracle_and_matches_golden(golden):
    g = golden("sample")
    geom = GridGeometry(tuple(g["origin"]), float(g["dx"]), g["field"].shape)
    ox = OxygenField(geom, OxygenParams(), boundary=(Boundary.NEUMANN,) * 3, device=DEV)
    ox.field.values.copy_(_t(g["field"]))
    pop = _pop_from(g["positions"])
    ox.sample_at_cells(pop)
    got = pop.oxygen_numpy()
    np.testing.assert_array_equal(got, orc.sample(orc.Geometry(geom.origin, geom.dx, geom.shape), g["field"], g["positions"]))
    np.testing.assert_allclose(got, g["expected"], rtol=1e-5, atol=1e-5)


def test_sampling_is_exact_for_linear_fields():
    geom = GridGeometry.centered_cube(200.0, 25.0)
    ox = OxygenField(geom, OxygenParams(), boundary=(Boundary.NEUMANN,) * 3, device=DEV)
    x, y, z = np.meshgrid(*geom.node_coordinates(), indexing="ij")
    ox.field.assign(3.0 + 0.1 * x - 0.05 * y + 0.02 * z)
    pos = np.random.default_rng(1).uniform(-90.0, 90.0, size=(200, 3)).astype(np.float32)
    pop = _pop_from(pos)
    ox.sample_at_cells(pop)
    np.testing.assert_allclose(pop.oxygen_numpy(), 3.0 + 0.1 * pos[:, 0] - 0.05 * pos[:, 1] + 0.02 * pos[:, 2], atol=1e-4)


# ---- SOR ------------------------------------------------------------------------------------------------------
def _oracle_params(field, kin, omega, has_source=0, source_k=1.0):
    g = field.geometry
    return orc.sor_params(orc.Geometry(g.origin, g.dx, g.shape), field.boundary_flags, field.boundary_value,
                          kin.diffusion, kin.uptake_max, kin.michaelis_k, omega, has_source, source_k)


@pytest.mark.parametrize("sweeps", [1, 7, 40])
def test_sor_sweeps_bitwise_equal_oracle_with_production_source_and_pins(sweeps):
    from warpbiocell_gb300.fields.diffusion import sor_chunk, sor_params

    geom = GridGeometry(origin=(0.0, 0.0, 0.0), dx=12.0, shape=(23, 19, 17))
    ox = OxygenField(geom, OxygenParams(boundary_value=30.0), boundary=MIXED, device=DEV)
    rng = np.random.default_rng(sweeps)
    pins = rng.random(geom.shape) < 0.03
    ox.field.set_fixed(pins)
    ox.field.assign(rng.uniform(0.0, 40.0, geom.shape).astype(np.float32))
    density = rng.uniform(0.0, 3e-3, geom.shape).astype(np.float32)
    production = rng.uniform(0.0, 30.0, geom.shape).astype(np.float32)
    source = rng.uniform(0.0, 5.0, geom.shape).astype(np.float32)
    kin = ox.species.kinetics
    start = ox.numpy()
    res = torch.zeros(1, dtype=torch.float32, device=DEV)
    p = sor_params(ox.field, kin, 1.8, 1, 0.04)
    sor_chunk(ox.field, _t(density), p, sweeps, res, _t(production), _t(source))
    values = start.copy()
    r_ref = orc.sor_sweeps(_oracle_params(ox.field, kin, 1.8, 1, 0.04), sweeps, pins.astype(np.int32), density, values,
                           production, source)
    np.testing.assert_array_equal(ox.numpy(), values)
    assert float(res.item()) == np.float32(r_ref)


def test_steady_state_matches_exact_discrete_solution(golden):
    g = golden("steady_state")
    geom = GridGeometry(origin=(0.0, 0.0, 0.0), dx=10.0, shape=(8, 7, 6))
    params = OxygenParams(diffusion_coefficient=2.0e3, uptake_max=5.0e4, michaelis_k=3.0, boundary_value=20.0)
    settings = SolverSettings(omega=1.5, tolerance=1e-5, max_sweeps=20000, check_every=10)
    ox = OxygenField(geom, params, settings, boundary=MIXED, device=DEV)
    ox.density.copy_(_t(g["density1"]))
    report = ox.solve_steady_state()
    assert report.converged
    np.testing.assert_allclose(ox.numpy(), g["exact1"], atol=2e-3)
    values = np.full(geom.shape, np.float32(20.0))
    sweeps, res, ok = orc.solve_steady_state(_oracle_params(ox.field, params.kinetics, 1.5), settings,
                                             np.zeros(geom.shape, np.int32), g["density1"], values)
    assert (report.sweeps, ok) == (sweeps, True) and report.residual == np.float32(res)
    np.testing.assert_array_equal(ox.numpy(), values)


def test_steady_state_field_within_1e5_relative_of_fp64():
    """The converged float32 field against an FP64 solve of the same discrete problem."""
    geom = GridGeometry.centered_cube(400.0, 20.0)
    settings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=4000, check_every=10)
    ox = OxygenField(geom, OxygenParams(), settings, device=DEV)
    x, y, z = np.meshgrid(*geom.node_coordinates(), indexing="ij")
    density = np.where(x**2 + y**2 + z**2 < 150.0**2, 2.4e-4, 0.0).astype(np.float32)
    ox.density.copy_(_t(density))
    ox.solve_steady_state()
    v64 = np.full(geom.shape, 38.0)
    orc.solve_steady_state(_oracle_params(ox.field, ox.species.kinetics, 1.8),
                           SolverSettings(omega=1.8, tolerance=1e-13, max_sweeps=20000, check_every=10),
                           np.zeros(geom.shape, np.int32), density.astype(np.float64), v64, fp64=True)
    rel = np.abs(ox.numpy() - v64) / np.maximum(np.abs(v64), 1.0)
    assert rel.max() < 1e-5, rel.max()


def test_warm_start_needs_one_check_and_uniform_stays_uniform():
    geom = GridGeometry.centered_cube(400.0, 20.0)
    ox = OxygenField(geom, OxygenParams(), SolverSettings(omega=1.8, tolerance=1e-5, check_every=10), device=DEV)
    x, y, z = np.meshgrid(*geom.node_coordinates(), indexing="ij")
    ox.density.copy_(_t(np.where(x**2 + y**2 + z**2 < 150.0**2, 2.4e-4, 0.0).astype(np.float32)))
    first, second = ox.solve_steady_state(), ox.solve_steady_state()
    assert first.converged and second.converged and first.sweeps > 20 and second.sweeps == 10
    flat = OxygenField(geom, OxygenParams(boundary_value=40.0), device=DEV)
    flat.solve_steady_state()
    np.testing.assert_array_equal(flat.numpy(), 40.0)


def test_deferred_solve_equals_waiting_solve():
    """A solve whose report is read later (wbc_sor_solve_deferred, as a cell step launches its
    field solves) gives the same field bits and report as the solve that waits for it, also when
    a second deferred solve of the same field is started before the first is read."""
    geom = GridGeometry.centered_cube(400.0, 20.0)
    x, y, z = np.meshgrid(*geom.node_coordinates(), indexing="ij")
    density = _t(np.where(x**2 + y**2 + z**2 < 150.0**2, 2.4e-4, 0.0).astype(np.float32))
    settings = SolverSettings(omega=1.8, tolerance=1e-6, check_every=10)
    waits = OxygenField(geom, OxygenParams(), settings, device=DEV)
    defers = OxygenField(geom, OxygenParams(), settings, device=DEV)
    for f in (waits, defers):
        f.density.copy_(density)
    want = [waits.solve_steady_state(), waits.solve_steady_state()]
    first = defers.solve_steady_state(defer=True)
    second = defers.solve_steady_state(defer=True)  # reads the first before reusing its record
    got = [first.result(), second.result()]
    assert got == want and defers.last_report == want[1]
    np.testing.assert_array_equal(defers.numpy(), waits.numpy())


# ---- mechanics ------------------------------------------------------------------------------------------------
def test_neighbor_counts_match_brute_force_and_positions_match_oracle(golden):
    g = golden("contact")
    params = ContactParams(stiffness=10.0, damping=1.0, max_radius=9.0, margin=0.5)
    pop = _pop_from(g["positions"], radii=g["radii"])
    grid = make_neighbor_grid(params, DEV)
    contact_substep(pop, grid, params, dt=0.0)
    np.testing.assert_array_equal(pop.neighbor_counts_numpy(), g["counts"])
    np.testing.assert_allclose(pop.velocity[: pop.count].cpu().numpy(), g["velocities"], atol=2e-4)
    ref = g["positions"].copy()
    pop = _pop_from(g["positions"], radii=g["radii"])
    for step in range(1, 21):
        contact_substep(pop, grid, params, dt=0.01)
        orc.contact_substep(ref, g["radii"], params.query_radius, 128, params.query_radius, params.rate, 0.01)
        np.testing.assert_array_equal(pop.positions_numpy(), ref)  # canonical order: same bits
        np.testing.assert_allclose(pop.positions_numpy(), g["trajectory"][step], atol=2e-3)


def test_mechanics_laws():
    # single cell stays put; isolated cells have no contacts; only the active prefix is indexed
    pos = np.array([[3.0, -2.0, 5.0]], np.float32)
    pop = _pop_from(pos)
    params = ContactParams(stiffness=10.0, damping=1.0, max_radius=8.0)
    relax_contacts(pop, make_neighbor_grid(params, DEV), params, dt=0.01, substeps=50)
    np.testing.assert_array_equal(pop.positions_numpy(), pos)
    pop = _pop_from(np.array([[0.0, 0, 0], [1.0, 0, 0]], np.float32), capacity=50)
    contact_substep(pop, make_neighbor_grid(params, DEV), params, dt=0.0)
    np.testing.assert_array_equal(pop.neighbor_counts_numpy(), [1, 1])
    # pair overlap decays as (1 - 2 rate dt)^n and the midpoint stays put
    pop = _pop_from(np.array([[0.0, 0, 0], [13.0, 0, 0]], np.float32))
    relax_contacts(pop, make_neighbor_grid(params, DEV), params, dt=0.01, substeps=15)
    x = pop.positions_numpy()
    assert 16.0 - np.linalg.norm(x[1] - x[0]) == pytest.approx(3.0 * (1.0 - 0.2) ** 15, rel=1e-3)
    np.testing.assert_allclose(x[0] + x[1], [13.0, 0.0, 0.0], atol=1e-4)
    # centre of mass conserved in a compressed cluster
    pos = spherical_cluster(1500, R, spacing_factor=0.85, jitter=0.2, seed=2)
    pop = _pop_from(pos)
    com = pos.astype(np.float64).mean(0)
    relax_contacts(pop, make_neighbor_grid(params, DEV), params, dt=0.01, substeps=100)
    np.testing.assert_allclose(pop.positions_numpy().astype(np.float64).mean(0), com, atol=1e-3)


def test_contact_displacement_within_1e5_um_of_fp64():
    pos = uniform_ball(50000, 300.0, seed=5)
    radii = np.clip(np.random.default_rng(5).normal(8.0, 0.8, 50000), 6, 10).astype(np.float32)
    params = ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0)
    pop = _pop_from(pos, radii=radii)
    grid = make_neighbor_grid(params, DEV)
    for _ in range(3):
        before = pop.positions_numpy()
        contact_substep(pop, grid, params, dt=0.1)
        after = pop.positions_numpy()
        p32 = before.copy()
        _, nc32 = orc.contact_substep(p32, radii, params.query_radius, 128, params.query_radius, params.rate, 0.1)
        np.testing.assert_array_equal(pop.neighbor_counts_numpy(), nc32)
        np.testing.assert_array_equal(after, p32)
        # FP64 re-run of the same step (its neighbour counts may differ at d == query_radius by
        # rounding; velocities only involve overlapping pairs, far inside that radius)
        p64 = before.astype(np.float64)
        vel64, _ = orc.contact_substep(p64, radii, params.query_radius, 128, params.query_radius, params.rate, 0.1,
                                       fp64=True)
        v32 = pop.velocity[: pop.count].cpu().numpy().astype(np.float64)
        assert np.abs(v32 * 0.1 - vel64 * 0.1).max() < 1e-5  # per-step displacement
        ulp = np.spacing(np.abs(before)).astype(np.float64)
        assert np.all(np.abs(after - (before + vel64 * 0.1)) <= 1e-5 + ulp)


# ---- lifecycle --------------------------------------------------------------------------------------------
def _lp(**kw):
    return LifecycleParams(**kw)


def _compare_pop(pop, sim):
    n = pop.count
    assert n == sim.count
    np.testing.assert_array_equal(pop.positions_numpy(), sim.position[:n])
    np.testing.assert_array_equal(pop.states_numpy(), sim.cell_state[:n])
    np.testing.assert_array_equal(pop.ages_numpy(), sim.age[:n])
    np.testing.assert_array_equal(pop.rng_numpy(), sim.rng_state[:n])
    np.testing.assert_array_equal(pop.neighbor_counts_numpy(), sim.neighbor_count[:n])
    np.testing.assert_array_equal(pop.oxygen_numpy(), sim.oxygen_local[:n])


@pytest.mark.parametrize("mode", ["rules", "network"])
def test_lifecycle_decide_scan_place_bitwise_equal_oracle(mode):
    n = 30000
    pos = uniform_ball(n, 400.0, seed=6)
    rng = np.random.default_rng(6)
    states = rng.integers(0, 4, n).astype(np.int32)
    pop = _pop_from(pos, states, capacity=3 * n, seed=6)
    sim = orc.OracleSim.from_numpy(pos, np.full(n, R), capacity=3 * n, seed=6, states=states)
    o2 = rng.uniform(0.0, 12.0, n).astype(np.float32)
    glc = rng.uniform(0.0, 6.0, n).astype(np.float32)
    nc = rng.integers(0, 12, n).astype(np.int32)
    flags = rng.integers(0, 16, n).astype(np.int32)
    for t, a in ((pop.oxygen_local, o2), (pop.glucose_local, glc), (pop.neighbor_count, nc), (pop.fate_flags, flags)):
        t[:n] = _t(a)
    sim.oxygen_local[:n], sim.glucose_local[:n], sim.neighbor_count[:n], sim.fate_flags[:n] = o2, glc, nc, flags
    params = _lp(division_rate=0.7, death_rate=0.05, anoxic_death_rate=0.5, inhibition_threshold=8,
                 hypoxia_threshold=5.0, death_threshold=1.0, glucose_threshold=4.0, glucose_death_threshold=0.5,
                 necrosis_requires_glucose=True, phenotype_model=mode, apoptosis_rate=0.3, necrosis_rate=2.0)
    created = lifecycle_step(pop, params, dt=1.0)
    sim.decide_lifecycle(params, 1.0)
    assert created == sim.commit_divisions(params) and created > 500
    _compare_pop(pop, sim)
    np.testing.assert_array_equal(pop.division_offset[:n].cpu().numpy(), sim.division_offset[:n])
    np.testing.assert_array_equal(pop.fate_flags_numpy(), sim.fate_flags[: pop.count])


def test_every_cell_divides_exactly_once_and_capacity_overflow_places_nothing():
    n = 300
    pos = spherical_cluster(n, R, spacing_factor=1.0, jitter=0.1, seed=0)
    pop = _pop_from(pos, capacity=3 * n)
    params = _lp(division_rate=1.0e3, inhibition_threshold=10**6)
    assert lifecycle_step(pop, params, dt=1.0) == n and pop.count == 2 * n
    x = pop.positions_numpy()
    np.testing.assert_allclose(np.linalg.norm(x[n:] - x[:n], axis=1), R, rtol=1e-5)
    np.testing.assert_allclose(0.5 * (x[n:] + x[:n]), pos, atol=1e-5)
    assert np.all(pop.ages_numpy()[:n] == 1.0) and np.all(pop.ages_numpy()[n:] == 0.0)
    assert np.all(pop.cell_state[2 * n:].cpu().numpy() == int(CellState.DEAD))
    pop = _pop_from(pos[:50], capacity=60)
    before = pop.positions_numpy()
    with pytest.raises(CapacityError):
        lifecycle_step(pop, params, dt=1.0)
    assert pop.count == 50
    np.testing.assert_array_equal(pop.positions_numpy(), before)
    assert np.all(pop.position[50:].cpu().numpy() == 0.0)


def test_certain_death_and_death_statistics():
    pop = _pop_from(spherical_cluster(100, R, seed=0), capacity=300)
    assert lifecycle_step(pop, _lp(division_rate=1e3, death_rate=1e3, inhibition_threshold=10**6), dt=1.0) == 0
    assert state_counts(pop)[CellState.DEAD] == 100
    n = 20000
    pop = _pop_from(np.zeros((n, 3), np.float32))
    lifecycle_step(pop, _lp(division_rate=0.0, death_rate=0.05, inhibition_threshold=10**6), dt=1.0)
    p = 1.0 - np.exp(-0.05)
    assert abs(state_counts(pop)[CellState.DEAD] / n - p) < 4.0 * np.sqrt(p * (1 - p) / n)


def test_contact_inhibition_makes_crowded_cells_quiescent():
    cluster = spherical_cluster(400, R, spacing_factor=1.0, jitter=0.05, seed=3)
    pos = np.vstack([cluster, [[500.0, 0, 0], [0, 500.0, 0], [0, 0, 500.0]]]).astype(np.float32)
    n = pos.shape[0]
    pop = _pop_from(pos, capacity=3 * n)
    contact = ContactParams(stiffness=10.0, damping=1.0, max_radius=R, margin=2.0)
    contact_substep(pop, make_neighbor_grid(contact, DEV), contact, dt=0.0)
    crowded = pop.neighbor_counts_numpy() >= 6
    assert crowded.sum() > 100 and (~crowded).sum() >= 3
    created = lifecycle_step(pop, _lp(division_rate=1e3, inhibition_threshold=6), dt=1.0)
    states = pop.states_numpy()[:n]
    assert np.all(states[crowded] == int(CellState.QUIESCENT)) and np.all(states[~crowded] == 0)
    assert created == int((~crowded).sum())


# ---- whole coupled step ----------------------------------------------------------------------------------------
def _coupled(seed=0, capacity=12000, n=3000, steps=6):
    pos = uniform_ball(n, 120.0, seed=seed)
    radii = np.clip(np.random.default_rng(seed).normal(8.0, 0.8, n), 6, 10).astype(np.float32)
    geom = GridGeometry.centered_cube(400.0, 20.0)
    settings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=2000, check_every=20)
    oparams = OxygenParams(diffusion_coefficient=7.2e6, uptake_max=5.54e7, michaelis_k=1.0, boundary_value=12.0)
    lifecycle = LifecycleParams(division_rate=0.2, death_rate=0.01, anoxic_death_rate=0.5, inhibition_threshold=14,
                                hypoxia_threshold=5.0, death_threshold=1.0)
    contact = ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0, wall_rate=4.0)
    stepping = TimeStepping(dt_cells=0.25, dt_mechanics=0.125)
    return pos, radii, geom, settings, oparams, lifecycle, contact, stepping


def test_coupled_cell_steps_bitwise_equal_oracle():
    pos, radii, geom, settings, oparams, lifecycle, contact, stepping = _coupled()
    pop = CellPopulation.from_numpy(pos, radii, capacity=12000, device=DEV, seed=0)
    ox = OxygenField(geom, oparams, settings, device=DEV)
    grid = make_neighbor_grid(contact, DEV)
    sim = orc.OracleSim.from_numpy(pos, radii, capacity=12000, seed=0)
    sp = orc.OracleSpecies(orc.Geometry(geom.origin, geom.dx, geom.shape), (0, 0, 0), 12.0, 7.2e6,
                           ox.species.uptake_max, 1.0, settings)
    for _ in range(6):
        rep = cell_step(pop, grid, lifecycle, contact, stepping, oxygen=ox)
        daughters, (sweeps, residual, ok) = orc.cell_step(sim, lifecycle, contact, stepping.dt_cells,
                                                          stepping.dt_mechanics, sp)
        assert rep.daughters == daughters and rep.field_sweeps == sweeps and rep.field_converged == ok
        assert rep.field_residual == np.float32(residual)
        np.testing.assert_array_equal(ox.numpy(), sp.values)
        _compare_pop(pop, sim)
    assert pop.count > 3000 and state_counts(pop)[CellState.HYPOXIC] > 0


def test_coupled_run_is_reproducible_and_independent_of_capacity():
    pos, radii, geom, settings, oparams, lifecycle, contact, stepping = _coupled(seed=1)
    snaps = []
    for capacity in (12000, 12000, 20000):
        pop = CellPopulation.from_numpy(pos, radii, capacity=capacity, device=DEV, seed=1)
        ox = OxygenField(geom, oparams, settings, device=DEV)
        grid = make_neighbor_grid(contact, DEV)
        for _ in range(4):
            cell_step(pop, grid, lifecycle, contact, stepping, oxygen=ox)
        snaps.append((pop.count, pop.positions_numpy(), pop.states_numpy(), ox.numpy()))
    for s in snaps[1:]:
        assert s[0] == snaps[0][0]
        for a, b in zip(s[1:], snaps[0][1:]):
            np.testing.assert_array_equal(a, b)


# ---- the shared-memory resident solver against the streaming colour launches and the oracle ------------
def _solve_with_path(path, geom, boundary, start, density, pins=None, production=None, source=None, settings=None,
                     tuning=None):
    from warpbiocell_gb300.fields import diffusion
    from warpbiocell_gb300.fields.diffusion import solve_steady_state
    from warpbiocell_gb300.fields.scalar_field import ScalarField
    from warpbiocell_gb300.fields.diffusion import UptakeKinetics

    f = ScalarField.create(geom, 30.0, boundary=boundary, device=DEV)
    if pins is not None:
        f.set_fixed(pins)
    f.assign(start)
    kin = UptakeKinetics(2.0e3, 5.0e4, 3.0)
    res = torch.zeros(1, dtype=torch.float32, device=DEV)
    old, old_tuning = diffusion.solver_path, diffusion.solver_tuning
    diffusion.solver_path, diffusion.solver_tuning = path, tuning
    try:
        rep = solve_steady_state(f, _t(density), kin, settings, res,
                                 production=None if production is None else _t(production),
                                 source=None if source is None else _t(source), source_k=0.04)
        info = dict(diffusion.last_solve)
    finally:
        diffusion.solver_path, diffusion.solver_tuning = old, old_tuning
    return f.numpy(), rep, info


@pytest.mark.parametrize("shape, boundary, extras", [
    ((37, 29, 23), MIXED, False),
    ((41, 41, 41), (Boundary.DIRICHLET,) * 3, False),
    ((33, 27, 31), (Boundary.NEUMANN, Boundary.DIRICHLET, Boundary.NEUMANN), True),
    ((97, 89, 101), (Boundary.DIRICHLET,) * 3, True),
])
def test_resident_solver_bitwise_equals_streaming_and_oracle(shape, boundary, extras):
    geom = GridGeometry(origin=(0.0, 0.0, 0.0), dx=10.0, shape=shape)
    rng = np.random.default_rng(sum(shape))
    start = rng.uniform(5.0, 30.0, shape).astype(np.float32)
    density = rng.uniform(0.0, 2.0e-3, shape).astype(np.float32)
    pins = (rng.random(shape) < 0.02) if extras else None
    production = rng.uniform(0.0, 40.0, shape).astype(np.float32) if extras else None
    source = rng.uniform(0.0, 5.0, shape).astype(np.float32) if extras else None
    settings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=300, check_every=20)
    a, ra, ia = _solve_with_path(1, geom, boundary, start, density, pins, production, source, settings)
    b, rb, ib = _solve_with_path(2, geom, boundary, start, density, pins, production, source, settings)
    assert ia["path"] == 1 and ib["path"] == 2 and ib["tiles"] >= 1
    assert (ra.sweeps, ra.converged, ra.residual) == (rb.sweeps, rb.converged, rb.residual)
    np.testing.assert_array_equal(a, b)
    # oracle: same start (Dirichlet faces / pins re-imposed as ScalarField.assign does)
    from warpbiocell_gb300.fields.scalar_field import ScalarField

    f = ScalarField.create(geom, 30.0, boundary=boundary, device=DEV)
    if pins is not None:
        f.set_fixed(pins)
    f.assign(start)
    values = f.numpy()
    p = orc.sor_params(orc.Geometry(geom.origin, geom.dx, geom.shape), f.boundary_flags, 30.0, 2.0e3, 5.0e4, 3.0, 1.8,
                       1 if source is not None else 0, 0.04)
    fixed = pins.astype(np.int32) if pins is not None else np.zeros(shape, np.int32)
    sweeps, residual, ok = orc.solve_steady_state(p, settings, fixed, density, values, production, source)
    assert (sweeps, ok) == (rb.sweeps, rb.converged) and np.float32(residual) == rb.residual
    np.testing.assert_array_equal(b, values)


@pytest.mark.parametrize("shape, boundary", [
    ((37, 29, 23), MIXED),
    ((33, 27, 31), (Boundary.NEUMANN, Boundary.DIRICHLET, Boundary.NEUMANN)),
    ((41, 41, 41), (Boundary.NEUMANN,) * 3),
])
def test_resident_tilings_bitwise(shape, boundary):
    """Every partition of the columns (tile count, strip count) gives the streaming path's bits:
    one strip, strips of one or two columns, tiles of a partial row, staircase tiles, and a chunk
    of 2 * 7 half-sweeps."""
    geom = GridGeometry(origin=(0.0, 0.0, 0.0), dx=10.0, shape=shape)
    rng = np.random.default_rng(7 + sum(shape))
    start = rng.uniform(5.0, 30.0, shape).astype(np.float32)
    density = rng.uniform(0.0, 2.0e-3, shape).astype(np.float32)
    pins = rng.random(shape) < 0.02
    production = rng.uniform(0.0, 40.0, shape).astype(np.float32)
    source = rng.uniform(0.0, 5.0, shape).astype(np.float32)
    settings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=63, check_every=7)
    a, ra, _ = _solve_with_path(1, geom, boundary, start, density, pins, production, source, settings)
    ny = shape[1]
    for tuning in [(0, 0), (0, 1), (0, 3), (17, 2), (40, 5), (7, 7), (2, 1), (3, 1), (60, ny), (100, ny // 2)]:
        b, rb, ib = _solve_with_path(2, geom, boundary, start, density, pins, production, source, settings,
                                     tuning=tuning)
        assert ib["path"] == 2, (tuning, ib)
        if tuning[0]:
            assert ib["tiles"] == tuning[0], (tuning, ib)
        if tuning[1]:
            assert ib["strips"] == tuning[1], (tuning, ib)
        assert (ra.sweeps, ra.converged, ra.residual) == (rb.sweeps, rb.converged, rb.residual), tuning
        np.testing.assert_array_equal(a, b, err_msg=str(tuning))


@pytest.mark.parametrize("shape, boundary", [
    ((21, 17, 301), MIXED),
    ((19, 22, 263), (Boundary.DIRICHLET,) * 3),
])
def test_resident_long_columns_bitwise(shape, boundary):
    """Columns of more than 128 entries per colour under several partitions."""
    geom = GridGeometry(origin=(0.0, 0.0, 0.0), dx=10.0, shape=shape)
    rng = np.random.default_rng(3 + sum(shape))
    start = rng.uniform(5.0, 30.0, shape).astype(np.float32)
    density = rng.uniform(0.0, 2.0e-3, shape).astype(np.float32)
    production = rng.uniform(0.0, 40.0, shape).astype(np.float32)
    settings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=40, check_every=10)
    a, ra, _ = _solve_with_path(1, geom, boundary, start, density, production=production, settings=settings)
    for tuning in [(0, 0), (8, 2), (30, 3), (60, 5)]:
        b, rb, ib = _solve_with_path(2, geom, boundary, start, density, production=production, settings=settings,
                                     tuning=tuning)
        assert ib["path"] == 2
        assert (ra.sweeps, ra.residual) == (rb.sweeps, rb.residual), tuning
        np.testing.assert_array_equal(a, b, err_msg=str(tuning))


def test_autotuned_solve_bitwise_equals_streaming():
    """The autotuner times candidate tunings on a scratch copy (the field is untouched) and the
    solve with its pick gives the streaming path's bits."""
    from warpbiocell_gb300.fields import diffusion

    shape = (45, 38, 41)
    geom = GridGeometry(origin=(0.0, 0.0, 0.0), dx=10.0, shape=shape)
    rng = np.random.default_rng(11)
    start = rng.uniform(5.0, 30.0, shape).astype(np.float32)
    density = rng.uniform(0.0, 2.0e-3, shape).astype(np.float32)
    settings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=120, check_every=20)
    a, ra, _ = _solve_with_path(1, geom, MIXED, start, density, settings=settings)
    diffusion.autotune_cache.clear()
    b, rb, ib = _solve_with_path(0, geom, MIXED, start, density, settings=settings, tuning=None)
    assert len(diffusion.autotune_cache) == 1
    (tiles, strips, us), = diffusion.autotune_cache.values()
    assert tiles >= 1 and strips >= 1 and us > 0.0
    assert (ib["path"], ib["tiles"], ib["strips"]) == (2, tiles, strips)
    assert (ra.sweeps, ra.converged, ra.residual) == (rb.sweeps, rb.converged, rb.residual)
    np.testing.assert_array_equal(a, b)


def test_resident_solver_runs_the_benchmark_grid():
    geom = GridGeometry.centered_cube(2400.0, 15.0)
    x, y, z = np.meshgrid(*geom.node_coordinates(), indexing="ij")
    density = np.where(x**2 + y**2 + z**2 < 1100.0**2, 1.5e-4, 0.0).astype(np.float32)
    start = np.full(geom.shape, 100.0, np.float32)
    settings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=100, check_every=20)
    a, ra, ia = _solve_with_path(1, geom, (Boundary.DIRICHLET,) * 3, start, density, settings=settings)
    b, rb, ib = _solve_with_path(2, geom, (Boundary.DIRICHLET,) * 3, start, density, settings=settings)
    assert ib["path"] == 2 and ib["tiles"] > 100
    assert (ra.sweeps, ra.residual) == (rb.sweeps, rb.residual)
    np.testing.assert_array_equal(a, b)


def test_adjoint_host_helpers():
    """The small kernels the adjoint's host code uses instead of eager torch operations: the
    fixed-order FP64 mean (the same bits on every call, within 1e-12 of numpy's), narrowing,
    filling, division and the compensated sum, each equal to its numpy counterpart."""
    rng = np.random.default_rng(31)
    st = _lib.stream(DEV)
    for n in (0, 1, 1000, 1_000_003):
        x = torch.from_numpy(rng.lognormal(0.0, 0.5, n).astype(np.float32)).to(DEV)
        scratch = torch.empty(257, dtype=torch.float64, device=DEV)
        _lib.call("wbc_mean", n, _lib.ptr(x), _lib.ptr(scratch), st)
        first = float(scratch[0].item())
        _lib.call("wbc_mean", n, _lib.ptr(x), _lib.ptr(scratch), st)
        assert float(scratch[0].item()) == first
        ref = float(x.cpu().numpy().astype(np.float64).mean()) if n else 0.0
        assert abs(first - ref) <= 1e-12 * max(1.0, abs(ref))
    n = 4099
    d = torch.from_numpy(rng.normal(0.0, 1e3, n)).to(DEV)
    f = torch.empty(n, dtype=torch.float32, device=DEV)
    _lib.call("wbc_narrow", n, _lib.ptr(d), _lib.ptr(f), st)
    np.testing.assert_array_equal(f.cpu().numpy(), d.cpu().numpy().astype(np.float32))
    _lib.call("wbc_fill", n, 38.5, _lib.ptr(f), st)
    assert bool((f == 38.5).all())
    a = torch.from_numpy(rng.lognormal(0.0, 1.0, n).astype(np.float32)).to(DEV)
    _lib.call("wbc_divide", n, _lib.ptr(a), 3.7, _lib.ptr(f), st)
    np.testing.assert_array_equal(f.cpu().numpy(), a.cpu().numpy() / np.float32(3.7))
    hi = torch.from_numpy(rng.uniform(-500, 500, n).astype(np.float32)).to(DEV)
    lo = torch.from_numpy((rng.uniform(-1, 1, n) * 1e-5).astype(np.float32)).to(DEV)
    x64 = torch.empty(n, dtype=torch.float64, device=DEV)
    pos = torch.empty(n, dtype=torch.float32, device=DEV)
    _lib.call("wbc_compensated_sum", n, _lib.ptr(hi), _lib.ptr(lo), _lib.ptr(x64), _lib.ptr(pos), st)
    want = hi.cpu().numpy().astype(np.float64) + lo.cpu().numpy().astype(np.float64)
    np.testing.assert_array_equal(x64.cpu().numpy(), want)
    np.testing.assert_array_equal(pos.cpu().numpy(), want.astype(np.float32))
    _lib.call("wbc_zero", _lib.ptr(pos), pos.numel() * 4, st)
    assert not pos.any()

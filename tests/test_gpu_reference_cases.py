"""The reference's own behavioural test cases run on the GPU path (reference tests
test_fields_numerical.py, test_neighbors.py, test_lifecycle.py, test_lifecycle_oxygen.py,
test_simulator.py and test_spheroid_biological.py): the same set-ups and the same pass criteria,
restated for torch tensors on cuda:0. Closed forms (the 1-D cosh profile of linear uptake, a
Gaussian pulse under the explicit scheme), symmetry and sign properties of the solver, edge cases
of the neighbour search, the oxygen rules of the lifecycle (statistical where the reference's
are), and the emergent behaviour of coupled spheroids."""

import numpy as np
import pytest
import torch

from warpbiocell_gb300.cells.initialization import spherical_cluster
from warpbiocell_gb300.cells.lifecycle import LifecycleParams, lifecycle_step
from warpbiocell_gb300.cells.mechanics import ContactParams, contact_substep, make_neighbor_grid
from warpbiocell_gb300.cells.model import CellState
from warpbiocell_gb300.cells.state import CellPopulation
from warpbiocell_gb300.fields.diffusion import SolverSettings, max_stable_dt
from warpbiocell_gb300.fields.oxygen import OxygenField, OxygenParams
from warpbiocell_gb300.fields.scalar_field import Boundary, GridGeometry
from warpbiocell_gb300.metrics.population import population_summary, state_counts
from warpbiocell_gb300.simulation.simulator import TimeStepping, cell_step

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
R = 8.0
CERTAIN = 1.0e3
NO_INHIBITION = 10**6
DIRICHLET = (Boundary.DIRICHLET,) * 3


def _field(geom, params, omega=1.5, tol=1e-6, boundary=DIRICHLET, max_sweeps=20000):
    settings = SolverSettings(omega=omega, tolerance=tol, max_sweeps=max_sweeps, check_every=10)
    return OxygenField(geom, params, settings, boundary=boundary, device=DEV)


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), device=DEV)


# ---- fields (reference tests/test_fields_numerical.py) -----------------------------------------------
def test_zero_consumption_converges_to_boundary_value_from_zero():
    ox = _field(GridGeometry.centered_cube(300.0, 20.0), OxygenParams(boundary_value=38.0), omega=1.8)
    ox.density.zero_()
    ox.field.values.fill_(0.0)
    ox.field.apply_dirichlet()
    report = ox.solve_steady_state()
    assert report.converged
    assert np.abs(ox.numpy() - 38.0).max() < 1e-4


@pytest.mark.parametrize("omega", [1.0, 1.5, 1.9])
def test_one_dimensional_linear_uptake_matches_cosh_profile(omega):
    """Dirichlet in x, zero flux in y and z, uptake linear in O (K much larger than O):
    O(x) = O_b cosh(kappa x) / cosh(kappa L)."""
    half, nx = 200.0, 81
    geom = GridGeometry(origin=(-half, 0.0, 0.0), dx=2 * half / (nx - 1), shape=(nx, 3, 3))
    diffusion, kappa, km = 1.0e4, 3.0 / half, 1.0e9
    params = OxygenParams(diffusion_coefficient=diffusion, uptake_max=kappa**2 * diffusion * km, michaelis_k=km,
                          boundary_value=1.0)
    ox = _field(geom, params, omega=omega, tol=1e-5,
                boundary=(Boundary.DIRICHLET, Boundary.NEUMANN, Boundary.NEUMANN))
    ox.density.fill_(1.0)
    report = ox.solve_steady_state()
    x = geom.node_coordinates()[0]
    exact = np.cosh(kappa * x) / np.cosh(kappa * half)
    v = ox.numpy()
    assert report.converged
    # discretisation error about (kappa dx)^2 / 12 plus the solver's; a wrong stencil or boundary
    # treatment would be off by O(0.1)
    np.testing.assert_allclose(v[:, 1, 1], exact, atol=2e-3)
    np.testing.assert_allclose(v[:, 0, 0], v[:, 1, 1], atol=1e-6)


def test_gaussian_pulse_diffuses_analytically():
    """The explicit scheme against the free-space Gaussian (boundaries far away), and the
    second moment growing by 2 D dt per step."""
    n, dx, diffusion = 41, 1.0, 1.0
    geom = GridGeometry(origin=(-20.0, -20.0, -20.0), dx=dx, shape=(n, n, n))
    params = OxygenParams(diffusion_coefficient=diffusion, uptake_max=0.0, michaelis_k=1.0, boundary_value=0.0)
    ox = _field(geom, params)
    ox.density.zero_()
    x, y, z = np.meshgrid(*geom.node_coordinates(), indexing="ij")
    r2 = x**2 + y**2 + z**2
    sigma0 = 3.0
    ox.field.assign(np.exp(-r2 / (2 * sigma0**2)))
    dt = 0.5 * max_stable_dt(ox.field, params.kinetics)
    steps = 48
    for _ in range(steps):
        ox.explicit_step(dt)
    var = sigma0**2 + 2 * diffusion * steps * dt
    exact = (sigma0**2 / var) ** 1.5 * np.exp(-r2 / (2 * var))
    v = ox.numpy().astype(np.float64)
    assert np.abs(v - exact).max() < 0.01 * exact.max()
    assert (v * x**2).sum() / v.sum() == pytest.approx(var, rel=2e-3)


def test_uniform_field_stays_uniform_under_explicit_steps():
    ox = _field(GridGeometry.centered_cube(200.0, 20.0), OxygenParams(boundary_value=40.0))
    ox.density.zero_()
    for _ in range(20):
        ox.explicit_step(0.5 * max_stable_dt(ox.field, ox.params.kinetics))
    np.testing.assert_array_equal(ox.numpy(), 40.0)
    with pytest.raises(ValueError):
        ox.explicit_step(1.5 * max_stable_dt(ox.field, ox.params.kinetics))


def test_symmetric_consumption_gives_symmetric_field():
    geom = GridGeometry.centered_cube(400.0, 20.0)
    ox = _field(geom, OxygenParams(), omega=1.8, tol=1e-5)
    x, y, z = np.meshgrid(*geom.node_coordinates(), indexing="ij")
    ox.density.copy_(_t(np.where(x**2 + y**2 + z**2 < 120.0**2, 2.4e-4, 0.0)))
    report = ox.solve_steady_state()
    v = ox.numpy()
    assert report.converged
    for axis in range(3):
        np.testing.assert_allclose(v, np.flip(v, axis=axis), atol=1e-4)
    np.testing.assert_allclose(v, np.transpose(v, (1, 2, 0)), atol=1e-4)
    c = geom.shape[0] // 2
    assert v[c, c, c] < 0.75 * ox.params.boundary_value


def test_strong_uptake_keeps_field_non_negative():
    ox = _field(GridGeometry.centered_cube(300.0, 20.0), OxygenParams(uptake_max=1.0e12), omega=1.9, tol=1e-5)
    ox.density.fill_(1.0e-3)
    report = ox.solve_steady_state()
    v = ox.numpy()
    assert report.converged
    assert v.min() >= 0.0
    assert v[ox.field.interior_mask()].max() < 1.0


# ---- neighbours (reference tests/test_neighbors.py) ------------------------------------------------------
def _one_pass(pos, radii, params):
    pop = CellPopulation.from_numpy(pos, radii, device=DEV)
    contact_substep(pop, make_neighbor_grid(params, DEV), params, dt=0.0)  # dt = 0: positions unchanged
    return pop


def test_neighbor_counts_with_mixed_radii_match_brute_force():
    rng = np.random.default_rng(5)
    pos = spherical_cluster(400, radius=8.0, spacing_factor=1.0, jitter=0.2, seed=5)
    radii = rng.uniform(5.0, 10.0, size=400).astype(np.float32)
    params = ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0, margin=0.0)
    pop = _one_pass(pos, radii, params)
    p = pos.astype(np.float64)  # the reference's brute force: all pairs in float64
    d = np.linalg.norm(p[:, None, :] - p[None, :, :], axis=2)
    np.fill_diagonal(d, np.inf)
    expected = (d < params.query_radius).sum(1)
    np.testing.assert_array_equal(pop.neighbor_counts_numpy(), expected)


def test_isolated_cells_have_no_contacts():
    pos = np.array([[0.0, 0.0, 0.0], [100.0, 0.0, 0.0], [0.0, 100.0, 0.0]], dtype=np.float32)
    pop = _one_pass(pos, np.full(3, 8.0, np.float32), ContactParams(stiffness=1.0, damping=1.0, max_radius=8.0))
    assert np.all(pop.neighbor_counts_numpy() == 0)
    assert np.all(pop.velocity[:3].cpu().numpy() == 0.0)


# ---- lifecycle (reference tests/test_lifecycle.py, test_lifecycle_oxygen.py) -----------------------------
def _cluster(n, oxygen=None, capacity=None, states=None):
    pos = spherical_cluster(n, R, spacing_factor=1.0, jitter=0.1, seed=0)
    pop = CellPopulation.from_numpy(pos, np.full(n, R), capacity=capacity or 3 * n, device=DEV, states=states)
    if oxygen is not None:
        pop.oxygen_local[:n].copy_(_t(oxygen))
    return pop


def test_states_follow_oxygen_thresholds():
    n = 300
    oxygen = np.linspace(0.0, 40.0, n).astype(np.float32)
    pop = _cluster(n, oxygen)
    lifecycle_step(pop, LifecycleParams(division_rate=0.0, hypoxia_threshold=8.0, death_threshold=2.0,
                                        inhibition_threshold=NO_INHIBITION), dt=1.0)
    s = pop.states_numpy()
    np.testing.assert_array_equal(s[oxygen < 8.0], int(CellState.HYPOXIC))
    np.testing.assert_array_equal(s[oxygen >= 8.0], int(CellState.PROLIFERATIVE))


def test_hypoxia_takes_precedence_over_crowding():
    n = 100
    pop = _cluster(n, np.full(n, 1.0, np.float32))
    pop.neighbor_count[:n].fill_(50)
    created = lifecycle_step(pop, LifecycleParams(division_rate=CERTAIN, hypoxia_threshold=8.0, death_threshold=0.5,
                                                  inhibition_threshold=8), dt=1.0)
    assert created == 0
    assert state_counts(pop)[CellState.HYPOXIC] == n


def test_division_stops_below_death_threshold_and_ramps_in_between():
    n = 30_000
    oxygen = np.concatenate([np.full(n // 3, 1.0), np.full(n // 3, 5.0), np.full(n // 3, 20.0)]).astype(np.float32)
    pop = _cluster(n, oxygen, capacity=2 * n + 10)
    rate = 0.2
    lifecycle_step(pop, LifecycleParams(division_rate=rate, hypoxia_threshold=8.0, death_threshold=2.0,
                                        inhibition_threshold=NO_INHIBITION), dt=1.0)
    thirds = np.split(pop.divide_flag[:n].cpu().numpy(), 3)
    assert thirds[0].sum() == 0
    p_full = 1.0 - np.exp(-rate)
    p_half = 1.0 - np.exp(-rate * (5.0 - 2.0) / (8.0 - 2.0))
    for observed, p in ((thirds[1].mean(), p_half), (thirds[2].mean(), p_full)):
        assert abs(observed - p) < 4.0 * np.sqrt(p * (1 - p) / (n // 3))


def test_anoxic_death_rate_applies_only_below_threshold():
    n = 40_000
    oxygen = np.concatenate([np.full(n // 2, 1.0), np.full(n // 2, 30.0)]).astype(np.float32)
    pop = _cluster(n, oxygen)
    lifecycle_step(pop, LifecycleParams(division_rate=0.0, death_rate=0.0, anoxic_death_rate=0.5,
                                        hypoxia_threshold=8.0, death_threshold=2.0,
                                        inhibition_threshold=NO_INHIBITION), dt=1.0)
    s = pop.states_numpy()
    p = 1.0 - np.exp(-0.5)
    dead_low = np.mean(s[: n // 2] == int(CellState.DEAD))
    assert abs(dead_low - p) < 4.0 * np.sqrt(p * (1 - p) / (n // 2))
    assert np.all(s[n // 2:] != int(CellState.DEAD))


def test_daughter_inherits_oxygen_and_state():
    n = 50
    pop = _cluster(n, np.full(n, 5.0, np.float32))
    created = lifecycle_step(pop, LifecycleParams(division_rate=CERTAIN, hypoxia_threshold=8.0, death_threshold=2.0,
                                                  inhibition_threshold=NO_INHIBITION), dt=1.0)
    assert created == n
    assert np.all(pop.states_numpy() == int(CellState.HYPOXIC))
    np.testing.assert_array_equal(pop.oxygen_numpy(), 5.0)


def test_oxygen_independent_defaults_are_unchanged():
    n = 200
    pop = _cluster(n, np.zeros(n, np.float32))
    created = lifecycle_step(pop, LifecycleParams(division_rate=CERTAIN, inhibition_threshold=NO_INHIBITION), dt=1.0)
    assert created == n
    assert np.all(pop.states_numpy() == int(CellState.PROLIFERATIVE))


def test_dead_cells_neither_divide_nor_move_nor_age():
    n = 200
    states = np.full(n, int(CellState.PROLIFERATIVE), dtype=np.int32)
    dead = np.arange(0, n, 3)
    states[dead] = int(CellState.DEAD)
    pop = _cluster(n, capacity=3 * n, states=states)
    before = pop.positions_numpy()
    created = lifecycle_step(pop, LifecycleParams(division_rate=CERTAIN, death_rate=0.0,
                                                  inhibition_threshold=NO_INHIBITION), dt=1.0)
    assert created == n - dead.size
    assert pop.count == 2 * n - dead.size
    np.testing.assert_array_equal(pop.positions_numpy()[dead], before[dead])
    assert np.all(pop.states_numpy()[dead] == int(CellState.DEAD))
    assert np.all(pop.ages_numpy()[dead] == 0.0)
    assert np.all(pop.states_numpy()[n:] == int(CellState.PROLIFERATIVE))


# ---- full steps (reference tests/test_simulator.py) ------------------------------------------------------
def _run(seed, capacity, steps=12, n0=400):
    pos = spherical_cluster(n0, R, spacing_factor=1.0, jitter=0.1, seed=seed)
    pop = CellPopulation.from_numpy(pos, np.full(n0, R), capacity=capacity, device=DEV, seed=seed)
    contact = ContactParams(stiffness=10.0, damping=1.0, max_radius=R, margin=2.0)
    grid = make_neighbor_grid(contact, DEV)
    lifecycle = LifecycleParams(division_rate=0.2, death_rate=0.01, inhibition_threshold=8)
    stepping = TimeStepping(dt_cells=0.25, dt_mechanics=0.025)
    for _ in range(steps):
        cell_step(pop, grid, lifecycle, contact, stepping)
    return pop


def test_daughters_get_separated_by_mechanics():
    pop = _run(seed=1, capacity=4000, steps=4)
    x = pop.positions_numpy().astype(np.float64)
    d = np.linalg.norm(x[:, None, :] - x[None, :, :], axis=2)
    np.fill_diagonal(d, np.inf)
    assert (2.0 * R - d).max() < 0.35 * R


def test_metrics_are_consistent_and_seeds_differ():
    pop = _run(seed=2, capacity=4000)
    counts = state_counts(pop)
    summary = population_summary(pop)
    assert sum(counts.values()) == pop.count == summary["cells"]
    assert summary["living_cells"] + summary["dead_cells"] == pop.count
    assert counts[CellState.HYPOXIC] == 0
    assert summary["dead_cells"] > 0 and summary["proliferative_cells"] > 0
    assert summary["spheroid_radius"] > 50.0
    a, b = _run(seed=5, capacity=4000), _run(seed=6, capacity=4000)
    assert a.count != b.count or not np.array_equal(a.positions_numpy()[:400], b.positions_numpy()[:400])


# ---- emergent behaviour (reference tests/test_spheroid_biological.py) -----------------------------------
def _static_spheroid(n):
    pos = spherical_cluster(n, R, spacing_factor=1.0, jitter=0.1, seed=0)
    pop = CellPopulation.from_numpy(pos, np.full(n, R), device=DEV)
    ox = OxygenField(GridGeometry.centered_cube(800.0, 20.0), OxygenParams(),
                     SolverSettings(omega=1.8, tolerance=1e-5, check_every=10), device=DEV)
    ox.update(pop)
    return pop, ox


def test_large_spheroid_has_radial_gradient_and_hypoxic_core():
    pop, _ = _static_spheroid(12_000)
    x = pop.positions_numpy()
    r = np.linalg.norm(x, axis=1)
    o = pop.oxygen_numpy()
    assert o[r > r.max() - 30.0].mean() > 5.0 * o[r < 40.0].mean()
    assert np.mean(o < 8.0) > 0.3
    bins = np.linspace(0.0, r.max(), 10)
    profile = np.array([o[(r >= lo) & (r < hi)].mean() for lo, hi in zip(bins[:-1], bins[1:])])
    assert np.all(np.diff(profile) >= -1e-3)


def test_small_spheroid_is_fully_oxygenated():
    pop, _ = _static_spheroid(800)
    o = pop.oxygen_numpy()
    assert o.min() > 8.0 and o.min() < o.max()


def test_growing_spheroid_develops_hypoxia_and_keeps_a_viable_rim():
    n0 = 3000
    pos = spherical_cluster(n0, R, spacing_factor=1.0, jitter=0.1, seed=1)
    pop = CellPopulation.from_numpy(pos, np.full(n0, R), capacity=40_000, device=DEV, seed=1)
    contact = ContactParams(stiffness=10.0, damping=1.0, max_radius=R, margin=2.0)
    grid = make_neighbor_grid(contact, DEV)
    lifecycle = LifecycleParams.oxygen_dependent(division_rate=0.08, inhibition_threshold=8)
    stepping = TimeStepping(dt_cells=0.5, dt_mechanics=0.05)
    ox = OxygenField(GridGeometry.centered_cube(900.0, 20.0), OxygenParams(),
                     SolverSettings(omega=1.8, tolerance=1e-5, check_every=10), device=DEV)
    for _ in range(40):  # 20 h
        assert cell_step(pop, grid, lifecycle, contact, stepping, oxygen=ox).field_converged
    counts = state_counts(pop)
    x = pop.positions_numpy()
    r = np.linalg.norm(x - x.mean(axis=0), axis=1)
    s = pop.states_numpy()
    outer, inner = r > np.percentile(r, 90), r < np.percentile(r, 20)
    assert pop.count > n0
    assert counts[CellState.HYPOXIC] > 0 and counts[CellState.DEAD] > 0
    assert np.mean(s[outer] == int(CellState.DEAD)) < 0.05
    assert np.mean(s[inner] != int(CellState.PROLIFERATIVE)) > 0.9
    assert np.mean(s[outer] == int(CellState.PROLIFERATIVE)) > np.mean(s[inner] == int(CellState.PROLIFERATIVE))


# ---- species (reference tests/test_species.py) ----------------------------------------------------------
def _mixed_population(n, hypoxic_fraction=0.4, seed=1):
    pos = spherical_cluster(n, R, spacing_factor=1.0, jitter=0.1, seed=seed)
    states = np.full(n, int(CellState.PROLIFERATIVE), dtype=np.int32)
    r = np.linalg.norm(pos, axis=1)
    states[r < np.quantile(r, hypoxic_fraction)] = int(CellState.HYPOXIC)
    states[::17] = int(CellState.DEAD)
    return CellPopulation.from_numpy(pos, np.full(n, R), device=DEV, states=states)


def _glucose_lactate(glucose_boundary=5.0):
    from warpbiocell_gb300.fields.species import SpeciesParams

    glucose = SpeciesParams("glucose", "mM", diffusion=2.4e5, michaelis_k=0.04, boundary_value=glucose_boundary,
                            uptake_max=(3.0e4, 3.0e4, 4.5e5, 0.0))
    lactate = SpeciesParams("lactate", "mM", diffusion=2.4e5, michaelis_k=1.0, boundary_value=1.0,
                            production=(0.0, 0.0, 9.0e5, 0.0), production_source="glucose")
    return glucose, lactate


def test_per_state_densities_conserve_cells_and_combine_with_state_factors():
    from warpbiocell_gb300.fields.densities import CellDensities

    pop = _mixed_population(500)
    geom = GridGeometry.centered_cube(400.0, 20.0)
    densities = CellDensities(geom, device=DEV)
    densities.deposit(pop)
    dens = densities.numpy()
    assert abs(densities.total_numpy().sum() * geom.voxel_volume - 500) < 1e-3
    out = OxygenField(geom, OxygenParams(), device=DEV, densities=densities, uptake_state_factors={"hypoxic": 0.5})
    out.combine()
    np.testing.assert_allclose(out.density.cpu().numpy(), dens[0] + dens[1] + 0.5 * dens[2], rtol=1e-6, atol=1e-9)


def test_species_chain_consumes_glucose_and_produces_lactate():
    from warpbiocell_gb300.fields.metabolism import MetabolicFields

    geom = GridGeometry(origin=(-60.0, -60.0, -60.0), dx=15.0, shape=(9, 9, 9))
    pop = _mixed_population(150, hypoxic_fraction=0.5, seed=4)
    settings = SolverSettings(omega=1.5, tolerance=1e-6, max_sweeps=50000, check_every=10)
    fields = MetabolicFields(geom, OxygenParams(), list(_glucose_lactate()), settings, device=DEV)
    report = fields.update(pop)
    assert report.converged and set(report.reports) == {"oxygen", "glucose", "lactate"}
    assert fields["glucose"].numpy().min() < 4.9
    assert fields["lactate"].numpy().max() > 1.05
    assert pop.glucose_numpy().min() < 5.0 and pop.local_numpy("lactate").max() > 1.0


def test_no_glycolytic_cells_means_no_lactate_and_no_glucose_means_no_production():
    from warpbiocell_gb300.fields.metabolism import MetabolicFields

    geom = GridGeometry.centered_cube(300.0, 20.0)
    glucose, lactate = _glucose_lactate()
    pos = spherical_cluster(300, R, seed=2)
    pop = CellPopulation.from_numpy(pos, np.full(300, R), device=DEV)  # all proliferative
    fields = MetabolicFields(geom, OxygenParams(), [glucose, lactate], device=DEV)
    fields.update(pop)
    np.testing.assert_allclose(fields["lactate"].numpy(), 1.0, atol=1e-6)
    starved, _ = _glucose_lactate(glucose_boundary=0.0)
    fields = MetabolicFields(geom, OxygenParams(), [starved, lactate], device=DEV)
    fields.update(_mixed_population(300, hypoxic_fraction=1.0, seed=2))
    np.testing.assert_allclose(fields["lactate"].numpy(), 1.0, atol=1e-6)


def test_metabolic_fields_validate_species_order_and_names():
    from warpbiocell_gb300.fields.metabolism import MetabolicFields
    from warpbiocell_gb300.fields.species import SpeciesField, SpeciesParams

    geom = GridGeometry.centered_cube(200.0, 20.0)
    lactate = SpeciesParams("lactate", "mM", diffusion=1.0e5, michaelis_k=1.0, boundary_value=1.0,
                            production=(0.0, 0.0, 1.0, 0.0), production_source="glucose")
    with pytest.raises(ValueError, match="earlier species"):
        MetabolicFields(geom, OxygenParams(), [lactate], device=DEV)
    with pytest.raises(ValueError, match="duplicate"):
        MetabolicFields(geom, OxygenParams(), [SpeciesParams("oxygen", "mmHg", 1.0e5, 1.0, 1.0)], device=DEV)
    ox = OxygenField(geom, OxygenParams(), device=DEV)
    assert isinstance(ox, SpeciesField) and ox.name == "oxygen" and ox.species.unit == "mmHg"
    assert ox.params.boundary_value == 38.0 and ox.species.uptake_weights == (1.0, 1.0, 1.0, 0.0)


def test_lifecycle_glucose_rules():
    n = 400
    pos = spherical_cluster(n, R, seed=0)
    pop = CellPopulation.from_numpy(pos, np.full(n, R), capacity=3 * n, device=DEV)
    pop.oxygen_local[:n].fill_(1.0)  # anoxic everywhere; glucose for the first half only
    pop.glucose_local[: n // 2].fill_(5.0)
    pop.glucose_local[n // 2:n].fill_(0.1)
    lifecycle_step(pop, LifecycleParams(division_rate=0.0, anoxic_death_rate=1.0e3, hypoxia_threshold=8.0,
                                        death_threshold=2.0, glucose_threshold=4.0, glucose_death_threshold=0.5,
                                        necrosis_requires_glucose=True, inhibition_threshold=NO_INHIBITION), dt=1.0)
    s = pop.states_numpy()
    assert np.all(s[: n // 2] == int(CellState.HYPOXIC))  # anoxic but fed
    assert np.all(s[n // 2:] == int(CellState.DEAD))  # anoxic and starved
    # glucose ramps the division rate: none at 0.5 mM, full at 5 mM (oxygen ample)
    pop = CellPopulation.from_numpy(pos, np.full(n, R), capacity=3 * n, device=DEV)
    pop.oxygen_local[:n].fill_(30.0)
    pop.glucose_local[:n].fill_(0.5)
    params = LifecycleParams(division_rate=1.0e3, hypoxia_threshold=8.0, death_threshold=2.0, glucose_threshold=4.0,
                             glucose_death_threshold=0.5, inhibition_threshold=NO_INHIBITION)
    assert lifecycle_step(pop, params, dt=1.0) == 0
    pop.glucose_local[:n].fill_(5.0)
    assert lifecycle_step(pop, params, dt=1.0) == n


# ---- networks (reference tests/test_network.py) ----------------------------------------------------------
def _flags_population(n, flags, seed=0):
    pos = spherical_cluster(n, R, spacing_factor=1.0, jitter=0.1, seed=seed)
    pop = CellPopulation.from_numpy(pos, np.full(n, R), capacity=3 * n, device=DEV, seed=seed)
    pop.fate_flags[:n].copy_(torch.as_tensor(flags, dtype=torch.int32, device=DEV))
    return pop


def test_network_mode_divides_only_with_proliferation_on():
    n = 400
    flags = np.zeros(n, dtype=np.int32)
    flags[: n // 2] = 1  # proliferation
    flags[n // 4: n // 2] |= 4  # ... with growth arrest too
    pop = _flags_population(n, flags)
    created = lifecycle_step(pop, LifecycleParams(division_rate=1.0e3, inhibition_threshold=NO_INHIBITION,
                                                  phenotype_model="network"), dt=1.0)
    assert created == n // 4
    s = pop.states_numpy()[:n]
    assert np.all(s[: n // 4] == int(CellState.PROLIFERATIVE))
    assert np.all(s[n // 4:] == int(CellState.QUIESCENT))


def test_network_mode_death_rates_and_rules_mode_ignores_fates():
    n = 30000
    flags = np.zeros(n, dtype=np.int32)
    flags[: n // 3] = 2  # apoptosis
    flags[n // 3: 2 * n // 3] = 8  # necrosis
    pop = _flags_population(n, flags, seed=5)
    lifecycle_step(pop, LifecycleParams(division_rate=0.0, phenotype_model="network", apoptosis_rate=0.5,
                                        necrosis_rate=1.0e3), dt=1.0)
    dead = pop.states_numpy()[:n] == int(CellState.DEAD)
    assert abs(dead[: n // 3].mean() - (1.0 - np.exp(-0.5))) < 0.02
    assert dead[n // 3: 2 * n // 3].all() and not dead[2 * n // 3:].any()
    pop = _flags_population(200, np.full(200, 8, dtype=np.int32))  # necrosis everywhere, rules mode
    lifecycle_step(pop, LifecycleParams(division_rate=0.0, necrosis_rate=1.0e3), dt=1.0)
    assert not (pop.states_numpy()[:200] == int(CellState.DEAD)).any()


def test_microc_network_fates_follow_the_environment(golden):
    """The MicroC model: necrosis only without oxygen and glucose; under hypoxia with glucose the
    glycolytic switch keeps ATP up and proliferation unchanged."""
    from tests._networks import microc_network
    from warpbiocell_gb300.network.runtime import InputClamp, NetworkParams, NetworkRuntime

    net = microc_network(golden)
    n = 3000
    pos = spherical_cluster(n, R, spacing_factor=1.0, jitter=0.1, seed=8)
    pop = CellPopulation.from_numpy(pos, np.full(n, R), capacity=3 * n, device=DEV, seed=8)
    pop.local_field("lactate")  # zero lactate at every cell
    clamps = (InputClamp("Oxygen_supply", "oxygen", 15.7), InputClamp("Glucose_supply", "glucose", 4.0),
              InputClamp("MCT1_stimulus", "lactate", 1.5), InputClamp("EGFR_stimulus", "constant", 1.0),
              InputClamp("cMET_stimulus", "constant", 1.0), InputClamp("FGFR_stimulus", "constant", 1.0))
    rt = NetworkRuntime(NetworkParams(net, update="asynchronous", updates_per_step=400, inputs=clamps), pop.capacity,
                        device=DEV, species_names=("oxygen", "glucose", "lactate"))

    def run(o2, glc):
        pop.oxygen_local.fill_(o2)
        pop.glucose_local.fill_(glc)
        rt.initialize(pop)
        for _ in range(20):
            rt.step(pop, dt_h=0.25)
        counts = {k: v / n for k, v in rt.fate_counts(pop).items()}
        s = rt.states_numpy(pop)
        idx = net.index
        return counts, s[:, idx["glycoATP"]].mean(), s[:, idx["mitoATP"]].mean(), s[:, idx["ATP_Production_Rate"]].mean()

    normoxia, _, mito_n, _ = run(30.0, 5.0)
    hypoxia, glyco_h, mito_h, atp_h = run(5.0, 5.0)
    starved, _, _, atp_s = run(5.0, 1.0)
    assert normoxia["necrosis"] == 0.0
    assert 0.1 < normoxia["proliferation"] < 0.35 and 0.05 < normoxia["apoptosis"] < 0.35
    assert mito_h < 0.05 < mito_n and glyco_h > 0.9 and atp_h > 0.9
    assert abs(hypoxia["proliferation"] - normoxia["proliferation"]) < 0.08
    assert starved["necrosis"] > 0.95 and starved["proliferation"] < 0.02 and atp_s < 0.05


def test_maboss_network_dynamics_are_reproducible(golden):
    from tests._networks import microc_network
    from warpbiocell_gb300.network.runtime import InputClamp, NetworkParams, NetworkRuntime

    net = microc_network(golden, rates=True)
    runs = []
    for _ in range(2):
        pos = spherical_cluster(500, R, spacing_factor=1.0, jitter=0.1, seed=21)
        pop = CellPopulation.from_numpy(pos, np.full(500, R), capacity=1500, device=DEV, seed=21)
        rt = NetworkRuntime(NetworkParams(net, update="maboss", time_units_per_h=8.0,
                                          inputs=(InputClamp("EGFR_stimulus", "constant", 1.0),)),
                            pop.capacity, device=DEV)
        rt.initialize(pop)
        for _ in range(4):
            rt.step(pop, dt_h=0.25)
        runs.append(rt.states_numpy(pop))
    assert np.array_equal(runs[0], runs[1])
    assert runs[0].any(axis=0).sum() > 10  # the chain actually moved nodes

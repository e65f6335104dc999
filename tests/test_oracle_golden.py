"""The CPU oracle against the reference's own numpy references and closed forms (no GPU).

Golden vectors come from tests/golden/make_golden.py, which runs the reference's
src/warpbiocell/reference/*.py and network code. These tests pin the oracle before the GPU
parity tests trust it. Tolerances are those of the reference's own tests where it has them
(test_fields_computational.py, test_mechanics.py, test_network.py).
"""

import numpy as np
import pytest

from oracle import oracle as orc

DIRICHLET, NEUMANN = 0, 1


class Settings:
    def __init__(self, omega=1.5, tolerance=1e-5, max_sweeps=20000, check_every=10):
        self.omega, self.tolerance, self.max_sweeps, self.check_every = omega, tolerance, max_sweeps, check_every


def test_deposit_matches_reference_density_per_state(golden):
    g = golden("deposit")
    geom = orc.Geometry(tuple(g["origin"]), float(g["dx"]), tuple(int(x) for x in g["shape"]))
    acc = orc.deposit(geom, g["positions"], g["states"])
    dens, _ = orc.density_convert(geom, acc)
    # fixed-point quantisation is 2^-24 per weight (reference test: atol 1e-8)
    np.testing.assert_allclose(dens, g["density"], atol=1e-8)
    inside = (np.floor((g["positions"] - g["origin"]) / g["dx"]) >= 0).all(1) & (
        np.floor((g["positions"] - g["origin"]) / g["dx"]) + 1 < g["shape"]).all(1)
    assert abs(dens.astype(np.float64).sum() * float(g["dx"]) ** 3 - inside.sum()) < 1e-3
    assert inside.sum() < len(inside)  # the fixture holds cells outside the support


def test_deposit_is_exact_integer_sum_and_order_independent(golden):
    g = golden("deposit")
    geom = orc.Geometry(tuple(g["origin"]), float(g["dx"]), tuple(int(x) for x in g["shape"]))
    acc = orc.deposit(geom, g["positions"], g["states"])
    perm = np.random.default_rng(0).permutation(len(g["states"]))
    acc2 = orc.deposit(geom, g["positions"][perm], g["states"][perm])
    np.testing.assert_array_equal(acc, acc2)
    orc.set_threads(1)
    acc1 = orc.deposit(geom, g["positions"], g["states"])
    orc.set_threads(0)
    np.testing.assert_array_equal(acc, acc1)


def test_sample_matches_reference(golden):
    g = golden("sample")
    geom = orc.Geometry(tuple(g["origin"]), float(g["dx"]), g["field"].shape)
    got32 = orc.sample(geom, g["field"], g["positions"])
    got64 = orc.sample(geom, g["field"].astype(np.float64), g["positions"].astype(np.float64), fp64=True)
    np.testing.assert_allclose(got64, g["expected"], rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(got32, g["expected"], rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("fp64", [False, True])
def test_steady_state_matches_exact_discrete_solution(golden, fp64):
    g = golden("steady_state")
    geom = orc.Geometry((0.0, 0.0, 0.0), 10.0, (8, 7, 6))
    dt = np.float64 if fp64 else np.float32
    bc = (DIRICHLET, NEUMANN, DIRICHLET)
    p = orc.sor_params(geom, bc, 20.0, 2.0e3, 5.0e4, 3.0, 1.5)
    values = np.full(geom.shape, 20.0, dtype=dt)
    tol = 1e-12 if fp64 else 1e-5
    sweeps, res, ok = orc.solve_steady_state(p, Settings(tolerance=tol), np.zeros(geom.shape, np.int32),
                                             g["density1"].astype(dt), values, fp64=fp64)
    assert ok
    np.testing.assert_allclose(values, g["exact1"], atol=1e-8 if fp64 else 2e-3)


@pytest.mark.parametrize("fp64", [False, True])
def test_steady_state_with_production_and_source(golden, fp64):
    g = golden("steady_state")
    geom = orc.Geometry((0.0, 0.0, 0.0), 15.0, (9, 9, 9))
    dt = np.float64 if fp64 else np.float32
    p = orc.sor_params(geom, (DIRICHLET,) * 3, 1.0, 2.4e5, 3.0e4, 1.0, 1.5, has_source=1, source_k=0.04)
    values = np.full(geom.shape, 1.0, dtype=dt)
    tol = 1e-12 if fp64 else 1e-6
    _, _, ok = orc.solve_steady_state(p, Settings(tolerance=tol, max_sweeps=50000), np.zeros(geom.shape, np.int32),
                                      g["density2"].astype(dt), values, g["production2"].astype(dt),
                                      g["source2"].astype(dt), fp64=fp64)
    assert ok
    np.testing.assert_allclose(values, g["exact2"], atol=1e-8 if fp64 else 2e-3)
    assert g["exact2"].max() > 1.02  # production lifts the interior above the boundary value


def test_ftcs_matches_reference(golden):
    g = golden("steady_state")
    geom = orc.Geometry((0.0, 0.0, 0.0), 10.0, (7, 6, 5))
    p = orc.sor_params(geom, (DIRICHLET, NEUMANN, DIRICHLET), 20.0, 2.0e3, 5.0e4, 3.0, 1.0)
    p.dx2_over_D = np.float32(2.0e3 / 10.0**2)
    v = g["ftcs_values"].copy()
    fixed = np.zeros(geom.shape, np.int32)
    for step in range(1, 6):
        v = orc.ftcs_step(p, float(g["ftcs_dt"]), fixed, g["ftcs_density"], v)
        np.testing.assert_allclose(v, g["ftcs_steps"][step], rtol=1e-5, atol=1e-4)


def test_contact_counts_exact_and_velocities_match_reference(golden):
    g = golden("contact")
    for fp64 in (False, True):
        dt = np.float64 if fp64 else np.float32
        pos = g["positions"].astype(dt).copy()
        vel, nc = orc.contact_substep(pos, g["radii"], float(g["query_radius"]), 128, float(g["query_radius"]),
                                      float(g["rate"]), 0.0, fp64=fp64)
        np.testing.assert_array_equal(nc, g["counts"])
        np.testing.assert_allclose(vel, g["velocities"], atol=1e-9 if fp64 else 2e-4)
    assert g["counts"].max() >= 6


def test_contact_trajectory_matches_reference(golden):
    g = golden("contact")
    pos = g["positions"].copy()
    for step in range(1, 21):
        orc.contact_substep(pos, g["radii"], 18.5, 128, 18.5, 10.0, float(g["dt"]))
        np.testing.assert_allclose(pos, g["trajectory"][step], atol=2e-3)
    assert np.linalg.norm(g["trajectory"][-1] - g["positions"], axis=1).max() > 0.5


def test_contact_is_independent_of_bucket_dim_and_threads(golden):
    g = golden("contact")
    runs = []
    for dim, threads in ((128, 0), (7, 1), (3, 2)):
        orc.set_threads(threads)
        pos = g["positions"].copy()
        v, nc = orc.contact_substep(pos, g["radii"], 18.5, dim, 18.5, 10.0, 0.01)
        runs.append((pos, nc))
    orc.set_threads(0)
    for pos, nc in runs[1:]:
        np.testing.assert_array_equal(nc, runs[0][1])
        np.testing.assert_array_equal(pos, runs[0][0])  # same traversal order -> same bits


def test_network_sync_matches_reference_on_microc(golden):
    g = golden("network_microc")
    arrays = {k[5:]: g[k] for k in g.files if k.startswith("prog_")}
    n_nodes = len(g["names"])
    prog, keep = orc.program(arrays, n_nodes)
    words = np.ascontiguousarray(g["words"].astype(np.uint64))
    orc.lib().orc_network_update_sync(orc.ctypes.byref(prog), 256, 1, orc.P(words))
    np.testing.assert_array_equal(words, g["step1_words"])
    orc.lib().orc_network_update_sync(orc.ctypes.byref(prog), 256, 1, orc.P(words))
    np.testing.assert_array_equal(words, g["step2_words"])
    words = np.ascontiguousarray(g["words"].astype(np.uint64))
    orc.lib().orc_network_update_sync(orc.ctypes.byref(prog), 256, 2, orc.P(words))
    np.testing.assert_array_equal(words, g["step2_words"])


# ---- the project's random streams, exp and log -----------------------------------------------------
def test_streams_do_not_depend_on_capacity():
    a = orc.rng_init(5, 1000)
    b = orc.rng_init(5, 5000)
    np.testing.assert_array_equal(a, b[:1000])
    assert not np.array_equal(orc.rng_init(6, 1000), a)


def test_uniform_draws_are_uniform_and_independent():
    u = orc.rng_uniform(orc.rng_init(1, 20000), 16)
    assert u.min() >= 0.0 and u.max() < 1.0
    flat = u.ravel().astype(np.float64)
    assert abs(flat.mean() - 0.5) < 4 * np.sqrt(1 / 12 / flat.size)
    assert abs(flat.var() - 1 / 12) < 0.002
    hist, _ = np.histogram(flat, bins=64, range=(0, 1))
    expected = flat.size / 64
    chi2 = ((hist - expected) ** 2 / expected).sum()
    assert chi2 < 120  # 63 dof, p ~ 1e-5
    # neighbouring slots and consecutive draws are uncorrelated
    assert abs(np.corrcoef(u[:-1, 0], u[1:, 0])[0, 1]) < 0.03
    assert abs(np.corrcoef(u[:, 0], u[:, 1])[0, 1]) < 0.03


def test_exp_is_within_two_ulp():
    x = np.concatenate([np.linspace(-103.9, 88.7, 200001), -np.logspace(-8, 2, 20001), [0.0, -0.0]]).astype(np.float32)
    got = orc.expf(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    normal = ref > 1.2e-38
    ulp = np.spacing(ref[normal].astype(np.float32)).astype(np.float64)
    assert (np.abs(got[normal] - ref[normal]) / ulp).max() <= 2.0
    assert np.all(np.abs(got[~normal] - ref[~normal]) <= 1.5e-45)
    assert orc.expf(np.array([-1000.0, 1000.0, 0.0], np.float32)).tolist() == [0.0, float("inf"), 1.0]


def test_log_is_within_three_ulp():
    x = np.concatenate([np.logspace(-44, 38, 200001), np.linspace(0.5, 2.0, 10001)]).astype(np.float32)
    x = x[x > 0]
    got = orc.logf(x).astype(np.float64)
    ref = np.log(x.astype(np.float64))
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    ulp = np.maximum(ulp, np.spacing(np.float32(1e-7)))
    assert (np.abs(got - ref) / ulp).max() <= 3.0


def test_sphere_directions_are_unit_and_isotropic():
    d = orc.rng_sphere(orc.rng_init(3, 200000)).astype(np.float64)
    assert np.abs(np.linalg.norm(d, axis=1) - 1.0).max() < 3e-7
    assert np.abs(d.mean(axis=0)).max() < 0.01
    np.testing.assert_allclose((d**2).mean(axis=0), 1 / 3, atol=0.005)


# ---- lifecycle laws on the oracle (the reference's statistical tests, test_lifecycle.py:121-156) ------
class LP:
    def __init__(self, **kw):
        d = dict(division_rate=0.0289, death_rate=0.0, anoxic_death_rate=0.0, inhibition_threshold=8,
                 hypoxia_threshold=0.0, death_threshold=0.0, glucose_threshold=0.0, glucose_death_threshold=0.0,
                 necrosis_requires_glucose=False, placement_factor=1.0, phenotype_model="rules",
                 apoptosis_rate=0.0, necrosis_rate=0.0)
        d.update(kw)
        self.__dict__.update(d)


def test_oracle_branching_law_and_death_rate(golden):
    pos = golden("spherical_cluster")["c0"]
    sim = orc.OracleSim.from_numpy(np.tile(pos, (4, 1))[:2000], np.full(2000, 8.0), capacity=25000, seed=0)
    rate, dt, steps = 0.1, 1.0, 20
    params = LP(division_rate=rate, inhibition_threshold=10**6)
    counts = [sim.count]
    for _ in range(steps):
        sim.decide_lifecycle(params, dt)
        sim.commit_divisions(params)
        counts.append(sim.count)
    p = 1.0 - np.exp(-rate * dt)
    ratio = np.array(counts) / (2000 * (1.0 + p) ** np.arange(steps + 1))
    assert np.all(np.abs(ratio - 1.0) < 0.1) and abs(ratio[-1] - 1.0) < 0.07

    n = 20000
    sim = orc.OracleSim.from_numpy(np.zeros((n, 3), np.float32), np.full(n, 8.0), seed=0)
    params = LP(division_rate=0.0, death_rate=0.05, inhibition_threshold=10**6)
    sim.decide_lifecycle(params, 1.0)
    dead = (sim.cell_state[:n] == 3).sum()
    p = 1.0 - np.exp(-0.05)
    assert abs(dead / n - p) < 4.0 * np.sqrt(p * (1 - p) / n)


def test_oracle_every_cell_divides_once_into_its_slot(golden):
    pos = golden("spherical_cluster")["c3"]
    n = pos.shape[0]
    sim = orc.OracleSim.from_numpy(pos, np.full(n, 8.0), capacity=3 * n)
    params = LP(division_rate=1.0e3, inhibition_threshold=10**6)
    sim.decide_lifecycle(params, 1.0)
    assert sim.commit_divisions(params) == n
    parents, daughters = sim.position[:n], sim.position[n:2 * n]
    np.testing.assert_allclose(np.linalg.norm(daughters - parents, axis=1), 8.0, rtol=1e-5)
    np.testing.assert_allclose(0.5 * (daughters + parents), pos, atol=1e-5)
    assert np.all(sim.age[:n] == 1.0) and np.all(sim.age[n:2 * n] == 0.0)


def test_full_cell_steps_do_not_depend_on_the_thread_count():
    """The oracle is timed on one thread and on all host threads; both must give the same bits
    (contact per cell, exact integer deposit, red-black sweeps, max-residual, sequential scan)."""
    import math

    from warpbiocell_gb300.cells.initialization import clipped_normal_radii, uniform_ball
    from warpbiocell_gb300.cells.lifecycle import LifecycleParams
    from warpbiocell_gb300.cells.mechanics import ContactParams
    from warpbiocell_gb300.fields.diffusion import SolverSettings
    from warpbiocell_gb300.fields.oxygen import OxygenParams, species_params
    from warpbiocell_gb300.fields.scalar_field import GridGeometry

    n = 3000
    pos = uniform_ball(n, 180.0, seed=4)
    radii = clipped_normal_radii(n, 8.0, 0.8, 6.0, 10.0, seed=5)
    geom = GridGeometry.centered_cube(600.0, 20.0)
    og = orc.Geometry(geom.origin, geom.dx, geom.shape)
    s = species_params(OxygenParams(diffusion_coefficient=7.2e6, uptake_max=5.5385e7, michaelis_k=1.0,
                                    boundary_value=38.0))
    settings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=2000, check_every=20)
    contact = ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0, margin=0.0, wall_rate=4.0)
    lifecycle = LifecycleParams(division_rate=math.log(2.0) / 2.0, anoxic_death_rate=0.5, inhibition_threshold=8,
                                hypoxia_threshold=5.0, death_threshold=1.0)
    runs = []
    try:
        for threads in (1, 0):
            orc.set_threads(threads)
            sim = orc.OracleSim.from_numpy(pos, radii, capacity=3 * n, seed=7)
            species = [orc.OracleSpecies(og, (0, 0, 0), s.boundary_value, s.diffusion, s.uptake_max, s.michaelis_k,
                                         settings, production=s.production, name=s.name)]
            sim.contact_substep(contact.query_radius, 128, contact.query_radius, contact.rate, 0.0)
            orc.metabolic_update(sim, species, {})
            timings = {} if threads == 0 else None  # stage timing must not change the results
            daughters = [orc.full_cell_step(sim, lifecycle, contact, 0.1, 0.1, species, {}, timings=timings)[0]
                         for _ in range(3)]
            assert timings is None or set(timings) == {"fields", "network", "lifecycle", "mechanics"}
            m = sim.count
            runs.append((daughters, m, sim.position[:m].copy(), sim.cell_state[:m].copy(), sim.rng_state[:m].copy(),
                         sim.neighbor_count[:m].copy(), species[0].values.copy()))
    finally:
        orc.set_threads(0)
    one, many = runs
    assert sum(one[0]) > 0  # the steps divide cells
    assert one[0] == many[0] and one[1] == many[1]
    for a, b in zip(one[2:], many[2:]):
        np.testing.assert_array_equal(a, b)

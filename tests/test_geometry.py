"""Tissue-region host logic: shapes, signed distances on the grid, host sampling, seeding
(reference: tests/test_geometry.py, the parts that need no device)."""

import numpy as np
import pytest

from warpbiocell_gb300.fields.scalar_field import GridGeometry
from warpbiocell_gb300.geometry import CellBudgetError, Ellipsoid, Sphere, TissueRegion, Union, evaluate_on_grid
from warpbiocell_gb300.geometry.region import node_gradient

R = 8.0


def test_sphere_sdf_is_exact_on_nodes_and_volume_matches():
    geom = GridGeometry.centered_cube(400.0, 20.0)
    sphere = Sphere(radius=150.0)
    sdf = evaluate_on_grid(sphere, geom)
    x, y, z = np.meshgrid(*geom.node_coordinates(), indexing="ij")
    np.testing.assert_allclose(sdf, np.sqrt(x**2 + y**2 + z**2) - 150.0, atol=1e-4)
    region = TissueRegion(geom, sdf)
    assert abs(region.volume() / sphere.volume - 1.0) < 0.05


def test_ellipsoid_and_union_signs_and_bounds():
    ell = Ellipsoid(center=(10.0, 0.0, 0.0), radii=(200.0, 100.0, 50.0))
    x = np.array([10.0, 209.0, 211.0, 10.0, 10.0])
    y = np.array([0.0, 0.0, 0.0, 99.0, 101.0])
    d = ell.sdf(x, y, np.zeros(5))
    assert d[0] < 0 and d[1] < 0 and d[2] > 0 and d[3] < 0 and d[4] > 0
    assert abs(d[1] + 1.0) < 0.2 and abs(d[2] - 1.0) < 0.2
    lo, hi = ell.bounds
    np.testing.assert_allclose(lo, [-190.0, -100.0, -50.0])
    np.testing.assert_allclose(hi, [210.0, 100.0, 50.0])
    union = Union((Sphere(center=(-100.0, 0.0, 0.0), radius=80.0), Sphere(center=(100.0, 0.0, 0.0), radius=80.0)))
    d = union.sdf(np.array([-100.0, 100.0, 0.0]), np.zeros(3), np.zeros(3))
    assert d[0] == -80.0 and d[1] == -80.0 and d[2] == 20.0
    with pytest.raises(ValueError):
        Union(())
    with pytest.raises(ValueError):
        Sphere(radius=0.0)


def test_host_sampling_follows_the_analytical_distance():
    geom = GridGeometry.centered_cube(400.0, 20.0)
    region = TissueRegion.from_shape(Sphere(radius=150.0), geom)
    pts = np.random.default_rng(3).uniform(-180.0, 180.0, size=(300, 3))
    host = region.sample(pts)
    exact = np.linalg.norm(pts, axis=1) - 150.0
    assert np.abs(host - exact).max() < 0.15 * geom.dx
    np.testing.assert_array_equal(region.contains(pts), host < 0.0)


def test_node_gradient_is_the_unit_normal_of_a_sphere_away_from_the_centre():
    geom = GridGeometry.centered_cube(400.0, 20.0)
    sdf = evaluate_on_grid(Sphere(radius=150.0), geom)
    g = node_gradient(sdf, geom.dx)
    assert g.shape == sdf.shape + (3,) and g.dtype == np.float32
    x, y, z = np.meshgrid(*geom.node_coordinates(), indexing="ij")
    r = np.sqrt(x**2 + y**2 + z**2)
    sel = (r > 60.0) & (np.abs(x) < 180) & (np.abs(y) < 180) & (np.abs(z) < 180)
    np.testing.assert_allclose(np.linalg.norm(g[sel], axis=1), 1.0, atol=0.03)  # central differences of a cone


def test_fill_region_density_determinism_and_budget():
    from warpbiocell_gb300.geometry import fill_region

    geom = GridGeometry.centered_cube(600.0, 20.0)
    sphere = Sphere(radius=200.0)
    region = TissueRegion.from_shape(sphere, geom)
    a = fill_region(region, R, spacing_factor=1.0, jitter=0.1, seed=1)
    b = fill_region(region, R, spacing_factor=1.0, jitter=0.1, seed=1)
    np.testing.assert_array_equal(a, b)
    assert np.all(region.contains(a, margin=R))
    expected = sphere.volume / (2 * R) ** 3
    assert abs(a.shape[0] / expected - 1.0) < 0.15
    inner = fill_region(region, R, seed=1, within=Sphere(radius=100.0))
    assert 0 < inner.shape[0] < a.shape[0]
    assert np.all(np.linalg.norm(inner, axis=1) < 100.0)
    with pytest.raises(CellBudgetError, match="holds"):
        fill_region(region, R, seed=1, max_cells=100)


def test_wall_rate_stability_rule():
    from warpbiocell_gb300.cells.mechanics import ContactParams

    params = ContactParams(stiffness=1.0, damping=1.0, max_radius=R, wall_rate=40.0)
    with pytest.raises(ValueError, match="wall_rate"):
        params.check_substep(0.02)
    with pytest.raises(ValueError, match="wall_rate"):
        ContactParams(stiffness=1.0, damping=1.0, max_radius=R, wall_rate=-1.0)

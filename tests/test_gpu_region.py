"""Tissue-region confinement on the device against the oracle (reference: tests/test_geometry.py):
the contact substep with the region's wall push is bit-identical to the oracle's float32 restatement,
device sampling of the signed distance matches the host's, cells outside are pushed back in, a
compressed cluster stays inside the surface, and a field pinned outside the tissue gives the
oracle's bits."""

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from warpbiocell_gb300.cells.initialization import spherical_cluster, uniform_ball
from warpbiocell_gb300.cells.mechanics import ContactParams, contact_substep, make_neighbor_grid, relax_contacts
from warpbiocell_gb300.cells.state import CellPopulation
from warpbiocell_gb300.fields.diffusion import SolverSettings
from warpbiocell_gb300.fields.oxygen import OxygenField, OxygenParams
from warpbiocell_gb300.fields.scalar_field import GridGeometry
from warpbiocell_gb300.geometry import Ellipsoid, Sphere, TissueRegion, fill_region

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
R = 8.0


def _region(shape, side=400.0, dx=10.0):
    geom = GridGeometry.centered_cube(side, dx)
    return TissueRegion.from_shape(shape, geom, device=DEV), geom


def test_region_contact_substeps_bitwise_equal_oracle():
    region, geom = _region(Ellipsoid(center=(5.0, -3.0, 0.0), radii=(150.0, 110.0, 90.0)))
    pos = uniform_ball(3000, 140.0, seed=11)
    radii = np.random.default_rng(12).uniform(6.0, 9.0, size=pos.shape[0]).astype(np.float32)
    params = ContactParams(stiffness=10.0, damping=1.0, max_radius=9.0, wall_rate=20.0)
    pop = CellPopulation.from_numpy(pos, radii, device=DEV)
    grid = make_neighbor_grid(params, DEV)
    ref = pos.copy()
    rg = orc.Geometry(geom.origin, geom.dx, geom.shape)
    sdf, grad = region.sdf.cpu().numpy(), region.gradient.cpu().numpy()
    for _ in range(12):
        contact_substep(pop, grid, params, dt=0.02, region=region)
        vel, nc = orc.contact_substep_region(ref, radii, params.query_radius, 128, params.query_radius, params.rate,
                                             0.02, rg, sdf, grad, params.wall_rate)
        np.testing.assert_array_equal(pop.positions_numpy(), ref)
        np.testing.assert_array_equal(pop.velocity[: pop.count].cpu().numpy(), vel)
        np.testing.assert_array_equal(pop.neighbor_counts_numpy(), nc)


def test_device_sampling_matches_host_sampling():
    region, _ = _region(Sphere(radius=150.0), dx=20.0)
    pts = np.random.default_rng(4).uniform(-230.0, 230.0, size=(5000, 3)).astype(np.float32)  # some off the grid
    out = torch.empty(pts.shape[0], dtype=torch.float32, device=DEV)
    region.sample_at(torch.from_numpy(pts).to(DEV), pts.shape[0], out)
    np.testing.assert_allclose(out.cpu().numpy(), region.sample(pts), atol=2e-3)


def test_confinement_pushes_cells_back_inside():
    region, _ = _region(Sphere(radius=100.0), dx=20.0)
    pos = np.array([[130.0, 0.0, 0.0], [0.0, -120.0, 0.0], [0.0, 0.0, 0.0]], dtype=np.float32)
    pop = CellPopulation.from_numpy(pos, np.full(3, R, np.float32), device=DEV)
    params = ContactParams(stiffness=10.0, damping=1.0, max_radius=R, wall_rate=10.0)
    relax_contacts(pop, make_neighbor_grid(params, DEV), params, dt=0.02, substeps=100, region=region)
    x = pop.positions_numpy()
    r = np.linalg.norm(x, axis=1)
    assert r[0] < 100.0 - R + 0.5 and r[1] < 100.0 - R + 0.5  # whole sphere back within the tissue
    np.testing.assert_allclose(x[0] / r[0], [1.0, 0.0, 0.0], atol=1e-4)  # pushed radially
    np.testing.assert_array_equal(x[2], [0.0, 0.0, 0.0])  # untouched


def test_compressed_cluster_stays_confined_and_the_wall_acts():
    region, _ = _region(Sphere(radius=85.0), dx=20.0)
    pos = spherical_cluster(600, R, spacing_factor=0.85, jitter=0.2, seed=2)
    params = ContactParams(stiffness=10.0, damping=1.0, max_radius=R, wall_rate=10.0)
    pop = CellPopulation.from_numpy(pos, np.full(600, R, np.float32), device=DEV)
    relax_contacts(pop, make_neighbor_grid(params, DEV), params, dt=0.02, substeps=300, region=region)
    r = np.linalg.norm(pop.positions_numpy(), axis=1)
    assert r.max() < 85.0  # every centre inside the surface
    free = CellPopulation.from_numpy(pos, np.full(600, R, np.float32), device=DEV)
    relax_contacts(free, make_neighbor_grid(params, DEV), params, dt=0.02, substeps=300)
    assert np.linalg.norm(free.positions_numpy(), axis=1).max() > r.max() + 3.0


def test_seeded_region_stays_inside_under_relaxation():
    region, _ = _region(Sphere(radius=120.0))
    seeds = fill_region(region, R, spacing_factor=0.9, seed=3)
    params = ContactParams(stiffness=10.0, damping=1.0, max_radius=R, wall_rate=10.0)
    pop = CellPopulation.from_numpy(seeds, np.full(seeds.shape[0], R, np.float32), device=DEV)
    relax_contacts(pop, make_neighbor_grid(params, DEV), params, dt=0.02, substeps=200, region=region)
    assert seeds.shape[0] > 500
    assert region.sample(pop.positions_numpy()).max() < 0.0


def test_tissue_surface_oxygen_boundary_pins_outside_nodes():
    geom = GridGeometry(origin=(0.0, 0.0, 0.0), dx=10.0, shape=(9, 8, 8))
    region = TissueRegion.from_shape(Sphere(center=(40.0, 35.0, 35.0), radius=28.0), geom, device=DEV)
    params = OxygenParams(diffusion_coefficient=2.0e3, uptake_max=5.0e4, michaelis_k=3.0, boundary_value=20.0)
    settings = SolverSettings(omega=1.5, tolerance=1e-5, max_sweeps=20000, check_every=10)
    ox = OxygenField(geom, params, settings, device=DEV, fixed_outside=region)
    density = np.where(region.inside_mask(), 1.5e-3, 0.0).astype(np.float32)
    ox.density.copy_(torch.from_numpy(density).to(DEV))
    report = ox.solve_steady_state()
    outside = ~region.inside_mask()
    values = ox.numpy()
    assert report.converged
    np.testing.assert_array_equal(values[outside], 20.0)
    assert values[region.inside_mask()].min() < 20.0
    assert ox.field.interior_mask().sum() == region.inside_mask().sum()
    # the oracle's SOR from the same start with the same pins gives the same bits
    ref = np.full(geom.shape, 20.0, np.float32)
    p = orc.sor_params(orc.Geometry(geom.origin, geom.dx, geom.shape), ox.field.boundary_flags, 20.0,
                       params.diffusion_coefficient, params.uptake_max, params.michaelis_k, 1.5, 0, 0.0)
    sweeps, _, ok = orc.solve_steady_state(p, settings, outside.astype(np.int32), density, ref)
    assert ok and sweeps == report.sweeps
    np.testing.assert_array_equal(values, ref)

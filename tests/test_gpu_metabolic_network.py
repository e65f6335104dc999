"""GPU parity of the full coupled step with three species and a Boolean network per cell
(oxygen, glucose uptake coupled to it, lactate produced from glucose; a 106-node random
truth-table network clamped by oxygen and glucose; lifecycle in network mode): every cell array,
every field and every network word bit for bit against the oracle's mirror of
simulation/simulator.py:58-81 with fields/metabolism.py:99-111 and network/runtime.py:198-202."""

import numpy as np
import pytest

from oracle import oracle as orc
from warpbiocell_gb300.cells.initialization import clipped_normal_radii, uniform_ball
from warpbiocell_gb300.cells.lifecycle import LifecycleParams
from warpbiocell_gb300.cells.mechanics import ContactParams, make_neighbor_grid
from warpbiocell_gb300.cells.state import CellPopulation
from warpbiocell_gb300.fields.diffusion import SolverSettings
from warpbiocell_gb300.fields.metabolism import MetabolicFields
from warpbiocell_gb300.fields.oxygen import OxygenParams
from warpbiocell_gb300.fields.scalar_field import GridGeometry
from warpbiocell_gb300.fields.species import SpeciesParams, by_state
from warpbiocell_gb300.network.random_network import random_truth_table_network
from warpbiocell_gb300.network.runtime import InputClamp, NetworkParams, NetworkRuntime
from warpbiocell_gb300.simulation.simulator import TimeStepping, cell_step

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _setup(n=4000, ball=150.0, seed=3):
    pos = uniform_ball(n, ball, seed=seed)
    radii = clipped_normal_radii(n, seed=seed + 1)
    geom = GridGeometry.centered_cube(400.0, 20.0)
    settings = SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=2000, check_every=20)
    oxygen = OxygenParams(diffusion_coefficient=7.2e6, uptake_max=5.54e7, michaelis_k=1.0, boundary_value=12.0)
    glucose = SpeciesParams("glucose", "mM", diffusion=2.16e6, michaelis_k=0.04, boundary_value=5.0,
                            uptake_max=by_state(1.2e4))
    lactate = SpeciesParams("lactate", "mM", diffusion=2.88e6, michaelis_k=1.0, boundary_value=0.0,
                            production=by_state(2.4e4), production_source="glucose")
    net = random_truth_table_network(106, seed=seed)
    clamps = (InputClamp("Oxygen_supply", "oxygen", 5.0), InputClamp("Glucose_supply", "glucose", 2.0))
    lifecycle = LifecycleParams(division_rate=0.3, death_rate=0.01, anoxic_death_rate=0.5, inhibition_threshold=14,
                                hypoxia_threshold=5.0, death_threshold=1.0, phenotype_model="network",
                                apoptosis_rate=0.05, necrosis_rate=0.2)
    contact = ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0, wall_rate=4.0)
    stepping = TimeStepping(dt_cells=0.1, dt_mechanics=0.1)
    return pos, radii, geom, settings, oxygen, [glucose, lactate], net, clamps, lifecycle, contact, stepping


def test_metabolic_network_steps_bitwise_equal_oracle():
    pos, radii, geom, settings, oxygen, species, net, clamps, lifecycle, contact, stepping = _setup()
    n = pos.shape[0]
    capacity = 3 * n
    pop = CellPopulation.from_numpy(pos, radii, capacity=capacity, device=DEV, seed=3)
    fields = MetabolicFields(geom, oxygen, species, settings, device=DEV)
    rt = NetworkRuntime(NetworkParams(net, update="synchronous", updates_per_step=1, inputs=clamps), capacity,
                        device=DEV, species_names=tuple(fields.names))
    grid = make_neighbor_grid(contact, DEV)
    rt.initialize(pop)

    sim = orc.OracleSim.from_numpy(pos, radii, capacity=capacity, seed=3)
    og = orc.Geometry(geom.origin, geom.dx, geom.shape)
    osp = [orc.OracleSpecies(og, (0, 0, 0), f.species.boundary_value, f.species.diffusion, f.species.uptake_max,
                             f.species.michaelis_k, settings, production=f.species.production, name=name)
           for name, f in fields.species_fields.items()]
    src = {name: f.species.production_source for name, f in fields.species_fields.items() if f.species.production_source}
    clamp_tuples = tuple((net.index[c.node], {"oxygen": 0, "glucose": 1}[c.source], float(np.float32(c.threshold)),
                          1 if c.above else 0) for c in clamps)
    onet = orc.OracleNetwork({k: v.cpu().numpy() for k, v in rt._arrays.items()}, net.n_nodes, capacity,
                             clamps=clamp_tuples, fate_nodes=rt.fate_nodes, extra_names=tuple(rt.extra_names))
    onet.initialize(sim)
    np.testing.assert_array_equal(rt.words_numpy(pop), onet.words[:n])

    for _ in range(4):
        rep = cell_step(pop, grid, lifecycle, contact, stepping, oxygen=fields, network=rt)
        daughters, reports = orc.full_cell_step(sim, lifecycle, contact, stepping.dt_cells, stepping.dt_mechanics,
                                                osp, src, network=onet)
        assert rep.daughters == daughters
        assert rep.field_sweeps == sum(r[0] for r in reports)
        for (name, f), o in zip(fields.species_fields.items(), osp):
            np.testing.assert_array_equal(f.numpy(), o.values, err_msg=name)
        m = pop.count
        assert m == sim.count
        np.testing.assert_array_equal(rt.words_numpy(pop), onet.words[:m])
        np.testing.assert_array_equal(pop.fate_flags_numpy(), sim.fate_flags[:m])
        np.testing.assert_array_equal(pop.positions_numpy(), sim.position[:m])
        np.testing.assert_array_equal(pop.states_numpy(), sim.cell_state[:m])
        np.testing.assert_array_equal(pop.glucose_numpy(), sim.glucose_local[:m])
        np.testing.assert_array_equal(pop.local_numpy("lactate"), sim.local_field("lactate")[:m])
        np.testing.assert_array_equal(pop.rng_numpy(), sim.rng_state[:m])
    assert fields["lactate"].numpy().max() > 0.0 and fields["glucose"].numpy().min() < 5.0

"""Host-side logic of the drop-in API on CPU: initial conditions, network readers and compiler
against the reference's outputs (golden fixtures), parameter validation, and the refusal of a
CPU device (there is no CPU fallback). No GPU and no compute calls."""

import numpy as np
import pytest

from tests.conftest import GOLDEN
from warpbiocell_gb300.cells.initialization import spherical_cluster, uniform_ball
from warpbiocell_gb300.cells.lifecycle import LifecycleParams
from warpbiocell_gb300.cells.mechanics import ContactParams
from warpbiocell_gb300.fields.diffusion import SolverSettings, UptakeKinetics
from warpbiocell_gb300.fields.scalar_field import GridGeometry
from warpbiocell_gb300.fields.species import SpeciesParams, by_state
from warpbiocell_gb300.network import expression as ex
from warpbiocell_gb300.network.model import BooleanNetwork, NetworkError, Node, load_network, read_bnd, read_bnet
from warpbiocell_gb300.network.runtime import InputClamp, NetworkParams
from warpbiocell_gb300.simulation.simulator import TimeStepping


def test_spherical_cluster_matches_reference(golden):
    g = golden("spherical_cluster")
    for k in range(5):
        n, r, sp, jit, seed = g[f"c{k}_args"]
        got = spherical_cluster(int(n), float(r), spacing_factor=float(sp), jitter=float(jit), seed=int(seed))
        np.testing.assert_array_equal(got, g[f"c{k}"])


def test_uniform_ball_shape_and_support():
    p = uniform_ball(5000, 250.0, seed=0)
    r = np.linalg.norm(p, axis=1)
    assert p.dtype == np.float32 and p.shape == (5000, 3) and r.max() <= 250.0 + 1e-3
    assert abs(np.median(r) / 250.0 - 0.5 ** (1 / 3)) < 0.02


@pytest.mark.parametrize(
    "text, state, expected",
    [
        ("A & !B", {"A": 1, "B": 0}, True),
        ("A & !B", {"A": 1, "B": 1}, False),
        ("!(A | B) | C", {"A": 0, "B": 0, "C": 0}, True),
        ("A && B || !C", {"A": 1, "B": 1, "C": 1}, True),
        ("A AND NOT B", {"A": 1, "B": 0}, True),
        ("!!A", {"A": 1}, True),
        ("1", {}, True),
        ("A | 0", {"A": 0}, False),
    ],
)
def test_expression_parse_and_evaluate(text, state, expected):
    assert ex.evaluate(ex.parse(text), state) is expected


@pytest.mark.parametrize("text", ["A &", "(A | B", "A B", "& A", "A | )", "A # B", "3"])
def test_malformed_expressions_are_rejected(text):
    with pytest.raises(ex.ExpressionError):
        ex.parse(text)


def test_postfix_programs_match_reference_compiler(golden):
    g = golden("network_readers")
    index = {"A": 0, "B": 1, "C": 2, "a_1": 3, "B2": 4}
    for k, text in enumerate(g["exprs"]):
        ops, args = ex.compile_postfix(ex.parse(str(text)), index)
        np.testing.assert_array_equal(ops, g[f"e{k}_ops"])
        np.testing.assert_array_equal(args, g[f"e{k}_args"])
        assert ex.depth(ex.parse(str(text))) == int(g[f"e{k}_depth"])


def test_bnd_cfg_readers_match_reference(golden):
    g = golden("network_readers")
    net = read_bnd(GOLDEN / "toy_network.bnd", GOLDEN / "toy_network.cfg")
    assert net.names == [str(x) for x in g["names"]]
    assert net.input_names == [str(x) for x in g["inputs"]]
    np.testing.assert_allclose([n.p_on for n in net.nodes], g["p_on"])
    prog = net.programs()
    for key, value in prog.items():
        np.testing.assert_array_equal(value, g[f"prog_{key}"], err_msg=key)


def test_microc_programs_reproduce_reference_synchronous_steps(golden):
    """The MicroC programs exported by the reference evaluate (in the host reference semantics)
    to the reference's synchronous steps; the same arrays drive the GPU tests."""
    g = golden("network_microc")
    names = [str(x) for x in g["names"]]
    assert len(names) == 106 and len(g["input_names"]) == 25
    ops, args, start, length = g["prog_ops"], g["prog_args"], g["prog_start"], g["prog_length"]
    upd = set(g["prog_updatable"].tolist())
    assert len(upd) == 81 and length.max() <= 64
    for row, expected in zip(g["states"][:32], g["step1"][:32]):
        out = row.copy()
        for node in upd:
            stack = []
            for op, a in zip(ops[start[node]:start[node] + length[node]], args[start[node]:start[node] + length[node]]):
                if op == ex.OP_VAR:
                    stack.append(bool(row[a]))
                elif op == ex.OP_CONST:
                    stack.append(bool(a))
                elif op == ex.OP_NOT:
                    stack[-1] = not stack[-1]
                else:
                    b, a2 = stack.pop(), stack.pop()
                    stack.append((a2 and b) if op == ex.OP_AND else (a2 or b))
            out[node] = stack[0]
        np.testing.assert_array_equal(out, expected)


def test_microc_reader_on_reference_file_if_present(golden):
    import os
    from pathlib import Path

    root = os.environ.get("WBC_REFERENCE_ROOT")
    net_dir = Path(root or ".") / "configs" / "networks"
    if not root or not (net_dir / "microc_jaya.bnd").exists():
        pytest.skip("WBC_REFERENCE_ROOT does not name a checkout of the reference with its model files")
    net = load_network(net_dir / "microc_jaya.bnd", net_dir / "microc_jaya.cfg")
    g = golden("network_microc")
    assert net.names == [str(x) for x in g["names"]]
    for key, value in net.programs().items():
        np.testing.assert_array_equal(value, g[f"prog_{key}"], err_msg=key)


def test_pack_unpack_roundtrip_across_words(golden):
    g = golden("network_microc")
    nodes = [Node(str(n)) for n in g["names"]]
    net = BooleanNetwork(nodes)
    state = np.random.default_rng(1).random(net.n_nodes) < 0.5
    assert np.array_equal(net.unpack(net.pack(state)), state)
    np.testing.assert_array_equal(np.stack([net.pack(r) for r in g["states"][:8]]), g["words"][:8])


def test_bnet_reader_and_inputs(tmp_path):
    path = tmp_path / "toy.bnet"
    path.write_text("targets, factors\nI, I\nA, I\nB, A & !C\n# comment\nC, B\n")
    net = read_bnet(path)
    assert net.names == ["I", "A", "B", "C"] and net.input_names == ["I"] and net.n_words == 1


def test_network_errors(tmp_path):
    with pytest.raises(NetworkError):
        BooleanNetwork([Node("A", ex.parse("B"))])
    with pytest.raises(NetworkError):
        BooleanNetwork([Node("A"), Node("A")])
    with pytest.raises(NetworkError):
        load_network(tmp_path / "x.sbml")
    toy = BooleanNetwork([Node("I"), Node("A", ex.parse("I"))])
    with pytest.raises(NetworkError):
        NetworkParams(toy, inputs=(InputClamp("Z", "constant", 1.0),))
    with pytest.raises(NetworkError):
        NetworkParams(toy, update="random")
    with pytest.raises(NetworkError):
        NetworkParams(toy, outputs={"proliferation": "Z"})


def test_parameter_validation():
    with pytest.raises(ValueError):
        ContactParams(stiffness=0.0, damping=1.0, max_radius=8.0)
    params = ContactParams(stiffness=10.0, damping=1.0, max_radius=8.0)
    params.check_substep(0.04)
    with pytest.raises(ValueError):
        params.check_substep(0.1)
    with pytest.raises(ValueError):
        LifecycleParams(division_rate=-1.0)
    with pytest.raises(ValueError):
        LifecycleParams(inhibition_threshold=0)
    with pytest.raises(ValueError):
        LifecycleParams(placement_factor=0.0)
    with pytest.raises(ValueError):
        SolverSettings(omega=2.0)
    with pytest.raises(ValueError):
        UptakeKinetics(0.0, 1.0, 1.0)
    with pytest.raises(ValueError):
        GridGeometry(origin=(0, 0, 0), dx=0.0, shape=(4, 4, 4))
    assert TimeStepping(dt_cells=0.25, dt_mechanics=0.025).mechanics_substeps == 10
    with pytest.raises(ValueError):
        TimeStepping(dt_cells=0.1, dt_mechanics=0.2)
    geom = GridGeometry.centered_cube(400.0, 20.0)
    assert geom.shape == (21, 21, 21) and geom.origin == (-200.0, -200.0, -200.0)
    assert GridGeometry.centered_cube(2400.0, 15.0).shape == (161, 161, 161)


def test_species_helpers():
    assert by_state(None) == (0.0, 0.0, 0.0, 0.0)
    assert by_state(2.0) == (2.0, 2.0, 2.0, 0.0)
    assert by_state({"hypoxic": 3.0, "PROLIFERATIVE": 1.0}) == (1.0, 0.0, 3.0, 0.0)
    with pytest.raises(KeyError):
        by_state({"zombie": 1.0})
    s = SpeciesParams("glucose", "mM", 2.4e5, 0.04, 5.0, uptake_max=(3.0e4, 3.0e4, 4.5e5, 0.0))
    assert s.uptake_weights == (3.0e4 / 4.5e5, 3.0e4 / 4.5e5, 1.0, 0.0)


def test_cpu_device_is_refused():
    from warpbiocell_gb300 import _lib

    with pytest.raises(RuntimeError):
        _lib.resolve_device("cpu")


def _table_step(tables, updatable, row):
    out = row.copy()
    for node in updatable:
        k = int(tables["arity"][node])
        assert k >= 0
        idx = sum(int(row[tables["inputs"][6 * node + j]]) << j for j in range(k))
        out[node] = bool((int(tables["bits"][node]) >> idx) & 1)
    return out


def test_truth_tables_reproduce_reference_microc_steps_and_programs(golden):
    """Every MicroC node reads at most 5 nodes, so all 81 get truth tables; a step by table lookup
    reproduces the reference's synchronous steps, and on random states every table agrees with its
    program run with the kernels' postfix semantics (what the GPU evaluates either way)."""
    from warpbiocell_gb300.network.model import run_postfix, truth_tables

    g = golden("network_microc")
    ops, args, start, length = g["prog_ops"], g["prog_args"], g["prog_start"], g["prog_length"]
    upd = sorted(g["prog_updatable"].tolist())
    tables = truth_tables(ops, args, start, length, g["prog_updatable"], len(g["names"]))
    assert (tables["arity"][upd] >= 0).all()
    for row, expected in zip(g["states"], g["step1"]):
        np.testing.assert_array_equal(_table_step(tables, upd, row), expected)
    rng = np.random.default_rng(5)
    for _ in range(64):
        row = rng.random(len(g["names"])) < 0.5
        for node in upd:
            o = ops[start[node]:start[node] + length[node]].tolist()
            a = args[start[node]:start[node] + length[node]].tolist()
            values = {i: int(v) for i, v in enumerate(row)}
            assert _table_step(tables, [node], row)[node] == bool(run_postfix(o, a, values))


def test_truth_tables_of_random_networks_match_expressions():
    """Random 2-4 input truth-table networks: every updatable node gets a table equal to its DNF
    expression (the reference evaluator) on random states; the limit of 6 inputs is honoured."""
    from warpbiocell_gb300.network.random_network import random_truth_table_network

    net = random_truth_table_network(106, seed=3)
    arrays = net.programs()
    tables = net.truth_tables(arrays)
    upd = arrays["updatable"].tolist()
    assert (tables["arity"][upd] >= 0).all() and tables["arity"].max() <= 6
    rng = np.random.default_rng(11)
    for _ in range(64):
        row = rng.random(net.n_nodes) < 0.5
        np.testing.assert_array_equal(_table_step(tables, upd, row)[upd], net.targets(row)[upd])
    small = net.truth_tables(arrays, max_inputs=2)
    assert (small["arity"] <= 2).all() and (small["arity"] == -1).any()
    with pytest.raises(ValueError):
        net.truth_tables(arrays, max_inputs=7)


def test_population_rejects_bad_shapes_before_any_device_work():
    # reference: tests/test_state.py:21-27 (shape checks come before the device is resolved)
    from warpbiocell_gb300.cells.state import CellPopulation

    for pos, radii, kw in ((np.zeros((4, 2)), np.ones(4), {}), (np.zeros((4, 3)), np.ones(3), {}),
                           (np.zeros((4, 3)), np.ones(4), {"capacity": 2})):
        with pytest.raises(ValueError):
            CellPopulation.from_numpy(pos, radii, **kw)


def test_grid_geometry_helpers_and_solver_settings_validation():
    # reference: tests/test_fields_numerical.py:145-157
    from warpbiocell_gb300.fields.diffusion import SolverSettings
    from warpbiocell_gb300.fields.scalar_field import GridGeometry

    geom = GridGeometry.centered_cube(400.0, 20.0)
    assert geom.shape == (21, 21, 21)
    assert geom.origin == (-200.0, -200.0, -200.0) and geom.upper == (200.0, 200.0, 200.0)
    inside = geom.contains(np.array([[0.0, 0.0, 0.0], [199.0, -199.0, 0.0], [201.0, 0.0, 0.0]]))
    np.testing.assert_array_equal(inside, [True, True, False])
    with pytest.raises(ValueError):
        GridGeometry(origin=(0, 0, 0), dx=0.0, shape=(4, 4, 4))
    with pytest.raises(ValueError):
        SolverSettings(omega=2.0)


def test_explicit_step_refuses_an_unstable_dt():
    # reference: tests/test_fields_numerical.py:138-142 (checked before any device work)
    from types import SimpleNamespace

    from warpbiocell_gb300.fields.diffusion import UptakeKinetics, explicit_step, max_stable_dt
    from warpbiocell_gb300.fields.scalar_field import GridGeometry

    field = SimpleNamespace(geometry=GridGeometry.centered_cube(100.0, 20.0))
    kinetics = UptakeKinetics(diffusion=7.2e6, uptake_max=5.5e7, michaelis_k=1.0)
    limit = max_stable_dt(field, kinetics)
    assert limit == pytest.approx(20.0**2 / (6.0 * 7.2e6))
    with pytest.raises(ValueError, match="stability"):
        explicit_step(field, None, kinetics, 1.5 * limit, None)


def test_lifecycle_network_fields_and_time_step_are_validated():
    # reference: tests/test_network.py:364-368, tests/test_simulator.py:76-81
    for kw in ({"phenotype_model": "graph"}, {"apoptosis_rate": -1.0}, {"necrosis_rate": -1.0}):
        with pytest.raises(ValueError):
            LifecycleParams(**kw)
    with pytest.raises(ValueError):
        TimeStepping(dt_cells=0.0)


def test_device_module_refuses_the_cpu():
    # reference: device.py (resolve_device / cuda_available / synchronize); no CPU path here
    import torch

    from warpbiocell_gb300 import device

    assert device.cuda_available() == torch.cuda.is_available()
    with pytest.raises(RuntimeError):
        device.resolve_device("cpu")
    device.synchronize("cpu")  # nothing is queued on the host

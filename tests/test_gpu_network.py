"""GPU parity of the per-cell Boolean networks: the MicroC network's synchronous sweeps against
the reference's own synchronous_step (golden), and every update mode, clamp, fate packing and
inheritance against the oracle, bit for bit (reference tests: test_network.py:128-315 and the
bitwise CPU==CUDA checks of test_gpu.py:288-312)."""

import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.conftest import GOLDEN
from warpbiocell_gb300.cells.initialization import spherical_cluster
from warpbiocell_gb300.cells.lifecycle import LifecycleParams, lifecycle_step
from warpbiocell_gb300.cells.state import CellPopulation
from warpbiocell_gb300.network import expression as ex
from warpbiocell_gb300.network.model import BooleanNetwork, Node, read_bnd
from warpbiocell_gb300.network.runtime import InputClamp, NetworkParams, NetworkRuntime

from tests._networks import microc_network

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _population(n, seed=0, capacity=None):
    pos = spherical_cluster(n, 8.0, jitter=0.1, seed=seed)
    return CellPopulation.from_numpy(pos, np.full(n, 8.0), capacity=capacity, device=DEV, seed=seed)


def test_synchronous_kernel_matches_reference_on_microc(golden):
    g = golden("network_microc")
    net = microc_network(golden)
    pop = _population(256)
    rt = NetworkRuntime(NetworkParams(net, update="synchronous", updates_per_step=1), pop.capacity, device=DEV)
    rt.states.copy_(torch.as_tensor(g["words"].astype(np.uint64).view(np.int64), device=DEV))
    rt.update(pop, dt_h=0.25)
    np.testing.assert_array_equal(rt.words_numpy(pop), g["step1_words"])
    np.testing.assert_array_equal(rt.states_numpy(pop), g["step1"])
    rt.update(pop, dt_h=0.25)
    np.testing.assert_array_equal(rt.words_numpy(pop), g["step2_words"])
    rt.states.copy_(torch.as_tensor(g["words"].astype(np.uint64).view(np.int64), device=DEV))
    rt.update(pop, dt_h=0.25, updates_per_step=2)
    np.testing.assert_array_equal(rt.words_numpy(pop), g["step2_words"])


def _oracle_program(rt):
    return orc.program({k: v.cpu().numpy() for k, v in rt._arrays.items()}, rt.network.n_nodes)


@pytest.mark.parametrize("tables", [True, False], ids=["truth-tables", "programs"])
@pytest.mark.parametrize("mode, kw", [("synchronous", {"updates_per_step": 5}), ("asynchronous", {"updates_per_step": 300}),
                                      ("maboss", {"time_units_per_h": 8.0})])
def test_all_update_modes_bitwise_equal_oracle(golden, mode, kw, tables):
    """Both evaluation routes of the kernels (every MicroC node by its truth table, the runtime's
    default, or every node by running its postfix program) against the oracle's interpreter."""
    net = microc_network(golden)
    n = 4000
    pop = _population(n, seed=13)
    o = np.zeros(pop.capacity, dtype=np.float32)
    o[: n // 2] = 30.0
    g = np.full(pop.capacity, 5.0, dtype=np.float32)
    pop.oxygen_local.copy_(torch.as_tensor(o, device=DEV))
    pop.glucose_local.copy_(torch.as_tensor(g, device=DEV))
    clamps = (InputClamp(net.names[0], "oxygen", 15.7), InputClamp(net.names[1], "glucose", 4.0),
              InputClamp(net.names[2], "constant", 1.0), InputClamp(net.names[3], "glucose", 4.5, above=False))
    rt = NetworkRuntime(NetworkParams(net, update=mode, inputs=clamps, **kw), pop.capacity, device=DEV,
                        species_names=("oxygen", "glucose"))
    assert (rt._tables["arity"].cpu().numpy()[rt._arrays["updatable"].cpu().numpy()] >= 0).all()
    if not tables:
        rt.program.table_arity = rt.program.table_inputs = rt.program.table_bits = None
    rt.initialize(pop)
    # oracle mirror of initialize + 3 x step (clamp -> update -> fates)
    prog, keep = _oracle_program(rt)
    rng = orc.rng_init(13, n)
    words = np.zeros((n, net.n_words), dtype=np.uint64)
    lib = orc.lib()
    lib.orc_network_initialize(ctypes.byref(prog), n, orc.P(rt._arrays["p_on"].cpu().numpy()), orc.P(rng), orc.P(words))
    np.testing.assert_array_equal(rt.words_numpy(pop), words)
    c = {k: v.cpu().numpy() for k, v in rt._clamp.items()}
    fates = np.zeros(n, np.int32)
    for _ in range(3):
        rt.step(pop, dt_h=0.25)
        lib.orc_network_clamp_inputs(n, net.n_words, len(clamps), orc.P(c["node"]), orc.P(c["source"]),
                                     orc.P(c["threshold"]), orc.P(c["above"]), orc.P(o), orc.P(g), orc.P(o), orc.P(o),
                                     orc.P(words))
        if mode == "synchronous":
            lib.orc_network_update_sync(ctypes.byref(prog), n, kw["updates_per_step"], orc.P(words))
        elif mode == "asynchronous":
            lib.orc_network_update_async(ctypes.byref(prog), n, kw["updates_per_step"], orc.P(rng), orc.P(words))
        else:
            a = {k: rt._arrays[k].cpu().numpy() for k in ("rate_up_true", "rate_up_false", "rate_down_true", "rate_down_false")}
            lib.orc_network_update_maboss(ctypes.byref(prog), n, orc.f32(0.25 * kw["time_units_per_h"]), 20000,
                                          orc.P(a["rate_up_true"]), orc.P(a["rate_up_false"]),
                                          orc.P(a["rate_down_true"]), orc.P(a["rate_down_false"]), orc.P(rng),
                                          orc.P(words))
        lib.orc_network_read_fates(n, net.n_words, *rt.fate_nodes, orc.P(words), orc.P(fates))
        np.testing.assert_array_equal(rt.words_numpy(pop), words, err_msg=mode)
        np.testing.assert_array_equal(pop.fate_flags_numpy(), fates, err_msg=mode)
    np.testing.assert_array_equal(pop.rng_numpy(), rng)


def test_synchronous_toy_reaches_its_cycle():
    net = BooleanNetwork([Node("I"), Node("A", ex.parse("I")), Node("B", ex.parse("A & !C")), Node("C", ex.parse("B"))])
    pop = _population(8)
    rt = NetworkRuntime(NetworkParams(net, update="synchronous", updates_per_step=1,
                                      inputs=(InputClamp("I", "constant", 1.0),)), pop.capacity, device=DEV)
    rt.initialize(pop)
    seen = []
    for _ in range(8):
        rt.step(pop, dt_h=1.0)
        seen.append(tuple(rt.states_numpy(pop)[0].astype(int)))
    final = rt.states_numpy(pop)
    assert (final == final[0]).all() and seen[-1] == seen[-5] and seen[-1] != seen[-2]


def test_asynchronous_flip_probability_and_maboss_kinetics():
    net = BooleanNetwork([Node("I"), Node("A", ex.parse("I")), Node("B", ex.parse("A & !C")), Node("C", ex.parse("B"))])
    pop = _population(20000, seed=7)
    rt = NetworkRuntime(NetworkParams(net, update="asynchronous", updates_per_step=2,
                                      inputs=(InputClamp("I", "constant", 1.0),)), pop.capacity, device=DEV)
    rt.initialize(pop)
    rt.step(pop, dt_h=1.0)
    assert abs(rt.states_numpy(pop)[:, 1].mean() - (1.0 - (2.0 / 3.0) ** 2)) < 0.02
    r = 0.7
    net = BooleanNetwork([Node("X", ex.parse("1"), rate_up=(r, 0.0), rate_down=(0.0, 1.0))])
    pop = _population(40000, seed=11)
    rt = NetworkRuntime(NetworkParams(net, update="maboss", time_units_per_h=1.0), pop.capacity, device=DEV)
    rt.initialize(pop)
    t = 0.0
    for dt in (0.5, 0.5, 1.0):
        rt.update(pop, dt_h=dt)
        t += dt
        assert abs(rt.states_numpy(pop)[:, 0].mean() - (1.0 - np.exp(-r * t))) < 0.01


def test_fates_inheritance_and_reader_network():
    net = read_bnd(GOLDEN / "toy_network.bnd", GOLDEN / "toy_network.cfg")
    n = 200
    pop = _population(n, capacity=3 * n, seed=9)
    rt = NetworkRuntime(NetworkParams(net), pop.capacity, device=DEV)
    rt.initialize(pop)
    before = rt.states_numpy(pop).copy()
    flags_before = pop.fate_flags_numpy().copy()
    assert lifecycle_step(pop, LifecycleParams(division_rate=1.0e3, inhibition_threshold=10**6), dt=1.0) == n
    rt.inherit(pop, n)
    after = rt.states_numpy(pop)
    assert np.array_equal(after[:n], before) and np.array_equal(after[n:], before)
    assert np.array_equal(pop.fate_flags_numpy()[n:], flags_before)
    counts = rt.fate_counts(pop)
    assert counts["proliferation"] == int((after[:, net.index["Proliferation"]]).sum())
    assert counts["necrosis"] == 0 and counts["growth_arrest"] == 0

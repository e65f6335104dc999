"""The benchmark's synthetic workloads (host logic, no device): the seeded inputs have the shapes,
sizes and distributions of the configurations they stand in for, and the unit conversions match
the reference's parameters (per-hour rates, um, mmHg um^3/h uptake)."""

import math

import numpy as np
import pytest

import bench


def test_unit_conversions():
    # 2000 um^2/s -> um^2/h; 20 amol/s over an O2 solubility of 1.3e-21 mol/(um^3 mmHg) -> mmHg um^3/h
    assert bench.DIFFUSION == pytest.approx(7.2e6)
    assert bench.VMAX == pytest.approx(5.5385e7, rel=1e-4)
    assert bench.DT == pytest.approx(0.1)  # 6 min


@pytest.mark.parametrize("name, cells, ball", [("spheroid_10k_41", 10_000, 250.0), ("spheroid_100k_81", 100_000, 600.0)])
def test_cells_fill_the_ball_with_clipped_normal_radii(name, cells, ball):
    w = bench.WORKLOADS[name]
    pos, radii = bench.make_cells(w, seed=0)
    assert pos.shape == (cells, 3) and radii.shape == (cells,)
    r = np.linalg.norm(pos.astype(np.float64), axis=1)
    assert r.max() <= ball * (1 + 1e-6)
    # uniform in the ball: the fraction within half the radius is 1/8
    assert abs(np.mean(r < 0.5 * ball) - 0.125) < 0.02
    assert radii.min() >= 6.0 and radii.max() <= 10.0
    assert abs(radii.mean() - 8.0) < 0.05 and abs(radii.std() - 0.8) < 0.05
    pos2, radii2 = bench.make_cells(w, seed=0)
    assert np.array_equal(pos, pos2) and np.array_equal(radii, radii2)  # seeded


def test_headline_workload_matches_its_configuration():
    w = bench.WORKLOADS["spheroid_1M_161"]
    assert (w["cells"], w["ball_um"], w["dx_um"], w["boundary"]) == (1_000_000, 1200.0, 15.0, 100.0)
    P = bench.make_params(w)
    assert P["geom"].shape == (161, 161, 161) and P["geom"].dx == 15.0
    s = P["settings"]
    assert (s.omega, s.tolerance) == (1.8, 1e-6)
    assert P["contact"].query_radius == pytest.approx(20.0)  # 20 um hash cells
    assert P["stepping"].mechanics_substeps == 1
    assert P["lifecycle"].division_rate == pytest.approx(math.log(2.0) / 24.0)
    assert (P["lifecycle"].hypoxia_threshold, P["lifecycle"].death_threshold) == (5.0, 1.0)


def test_batched_sweep_instances_follow_the_sweep_definition():
    w = bench.WORKLOADS["batched_sweep_15"]
    specs = bench.batch_specs(w, seed=0)
    assert len(specs) == 15
    assert sorted({s["boundary"] for s in specs}) == [10.0, 20.0, 38.0, 60.0, 100.0]
    cells = np.array([s["cells"] for s in specs])
    assert cells.min() >= 2_000 and cells.max() <= 200_000 and len(set(cells.tolist())) > 10  # uneven
    nodes = np.array([s["nodes"] for s in specs])
    assert nodes.min() >= 41 and nodes.max() <= 121 and np.all(nodes % 2 == 1)
    for s in specs:  # the box spans 2.5 spheroid radii
        assert (s["nodes"] - 1) * s["dx"] == pytest.approx(2.5 * s["ball"], rel=1e-9)
    assert bench.batch_specs(w, seed=0) == specs  # seeded


def test_reference_arm_names_its_route_for_every_workload():
    import argparse

    for name in bench.WORKLOADS:
        out = bench.reference_unavailable(argparse.Namespace(workload=name))
        if bench.WORKLOADS[name].get("adjoint"):
            assert out["impl"] == "reference" and "warp-lang" in out["unavailable"]
        else:
            assert out is None  # timed by the C++ restatement


def test_host_cpu_record():
    host = bench.host_cpu()
    assert host["cpu_count"] >= 1 and host["machine"]
    assert host["model"] is None or isinstance(host["model"], str)


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` on the 10k-cell workload: one JSON line with the GPU arm's metric,
    unit and direction, a cpu_baseline describing the run and an e2e object with no copies."""
    import json
    import subprocess
    import sys

    out = subprocess.run([sys.executable, str(bench.ROOT / "bench.py"), "--impl", "reference", "--workload",
                          "spheroid_10k_41", "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                         timeout=600, check=True).stdout.strip().splitlines()
    assert len(out) == 1
    line = json.loads(out[0])
    assert line["impl"] == "reference" and line["metric"] == bench.metric_for("spheroid_10k_41")
    assert line["metric"] == "cell-steps/s @10k cells+41^3 O2 (coupled cell step)" and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True
    # the GPU arm's config object for the same workload, key for key
    assert line["config"] == bench.workload_config("spheroid_10k_41", 41 ** 3)
    assert line["value"] > 0 and line["steps"] == 1
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cpu = line["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["value"] == line["value"] and cpu["cores"] >= 1 and cpu["sample"]
    assert cpu["single_thread"]["cores"] == 1 and cpu["single_thread"]["value"] > 0
    stages = cpu["stages_ms_per_step"]
    assert set(stages) == {"fields", "network", "lifecycle", "mechanics"}
    assert sum(stages.values()) <= line["ms_per_step"] * 1.01 + 0.01
    assert cpu["host"]["cpu_count"] >= 1


@pytest.mark.parametrize("world", [2, 4, 8])
def test_batched_sweep_shards_cover_every_instance_and_balance(world):
    """The benchmark's batched sweep under torchrun: each rank batches its share of the 15 instances
    (greedy longest-first on cells + nodes^3); the shares are disjoint, cover every instance, and the
    busiest rank is within 5% of the mean load or holds a single instance that alone exceeds it."""
    from warpbiocell_gb300.simulation.sweep import partition_runs

    specs = bench.batch_specs(bench.WORKLOADS["batched_sweep_15"], seed=0)
    costs = [float(s["cells"] + s["nodes"] ** 3) for s in specs]
    shares = partition_runs(costs, world)
    assert len(shares) == world and all(shares)
    assert sorted(i for share in shares for i in share) == list(range(len(specs)))
    loads = [sum(costs[i] for i in share) for share in shares]
    assert max(loads) <= max(1.05 * sum(costs) / world, max(costs)) + 1e-9


def test_metric_labels_name_each_workload():
    assert bench.metric_for("spheroid_1M_161") == "cell-steps/s @1M cells+161^3 O2 (coupled cell step)"
    assert bench.metric_for("spheroid_100k_81") == "cell-steps/s @100k cells+81^3 O2 (coupled cell step)"
    assert "106-node networks" in bench.metric_for("metabolic_network_100k_81")
    assert "81^3" in bench.metric_for("metabolic_network_100k_81")
    assert "batched" in bench.metric_for("batched_sweep_15")
    assert "backward time" in bench.metric_for("adjoint_100k_81")

"""A sweep sharded by run over torch.distributed ranks (host logic, no device): the partition,
and two gloo ranks on the CPU that each run their share and gather the summary rows to rank 0.

The runs themselves need a GPU, so here each rank's run executor is replaced by a fake that
returns deterministic metrics; what is checked is which rank runs which configuration, that no
run is lost or repeated, and that the gathered summary equals the one-process summary.
"""

import csv
import math
import multiprocessing as mp
import os
import socket

import pytest

from warpbiocell_gb300.io.run_output import METRIC_COLUMNS
from warpbiocell_gb300.simulation import sweep as sw
from warpbiocell_gb300.simulation.experiment import RunResult

BASE = {
    "name": "sharding",
    "simulation": {"duration_h": 1.0, "dt_cells_h": 0.5, "dt_mechanics_h": 0.05},
    "cells": {"initial_count": 200, "max_cells": 5000},
    "oxygen": {"grid": {"box_um": 400.0, "dx_um": 20.0}},
    "output": {"metrics_every_h": 0.5, "figures": False},
}


def _spec():
    # uneven runs: the cell count and the grid spacing vary, so the costs differ
    return sw.SweepSpec(name="sharding", seeds=(0, 1),
                        grid={"cells.initial_count": [200, 800, 3000], "oxygen.grid.dx_um": [20.0, 10.0]})


def _fake_result(config) -> RunResult:
    n = config.cells.initial_count
    row = {c: 0.0 for c in METRIC_COLUMNS}
    row.update({"time_h": config.simulation.duration_h, "cells": n + config.simulation.seed,
                "spheroid_radius_um": float(n) ** (1.0 / 3.0)})
    return RunResult(status="completed", metrics=[row], wall_s=0.0)


def _fake_experiment(config, run_dir, device):
    _record(config)
    return _fake_result(config)


def _fake_batched(configs, run_dirs=None, device=None, log=None):
    for c in configs:
        _record(c)
    return [_fake_result(c) for c in configs]


def _record(config):
    path = os.environ.get("WBC_TEST_RAN")
    if path:
        with open(path, "a") as f:
            f.write(config.name + "\n")


def _worker(rank, world, port, out_dir, batched, ran_dir, queue):
    import torch.distributed as dist

    os.environ["WBC_TEST_RAN"] = os.path.join(ran_dir, f"rank{rank}.txt")
    sw._run_experiment = _fake_experiment
    sw.run_batched = _fake_batched
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        rows = sw.Sweep(_spec(), BASE).run(out_dir, batched=batched)
        queue.put((rank, rows))
    finally:
        dist.destroy_process_group()


def _same_rows(a: list[dict], b: list[dict], skip=()) -> bool:
    """Row lists equal value for value (NaN equals NaN: onsets that never happen are NaN)."""
    if len(a) != len(b):
        return False
    for ra, rb in zip(a, b):
        if set(ra) - set(skip) != set(rb) - set(skip):
            return False
        for k in ra:
            if k in skip:
                continue
            x, y = ra[k], rb[k]
            if isinstance(x, float) and isinstance(y, float) and math.isnan(x) and math.isnan(y):
                continue
            if x != y:
                return False
    return True


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_runs_covers_every_run_once_and_balances():
    costs = [5.0, 1.0, 4.0, 2.0, 3.0, 9.0, 0.5]
    for world in (1, 2, 3, 7, 9):
        parts = sw.partition_runs(costs, world)
        assert len(parts) == world
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        assert all(p == sorted(p) for p in parts)
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) <= sum(costs) / world + max(costs)  # greedy longest-first bound
        assert sw.partition_runs(costs, world) == parts  # deterministic
    assert sw.partition_runs([5.0, 1.0, 4.0, 2.0, 3.0, 9.0], 2) == [[4, 5], [0, 1, 2, 3]]
    with pytest.raises(ValueError):
        sw.partition_runs(costs, 0)


def test_run_cost_counts_cell_steps_and_node_steps():
    spec = _spec()
    configs = [sw.build_run_config(BASE, spec, label, values) for label, values in spec.runs()]
    small = [c for c in configs if c.cells.initial_count == 200 and c.oxygen.grid.dx_um == 20.0][0]
    # 2 steps x (200 cells + 21^3 nodes)
    assert sw.run_cost(small) == 2.0 * (200 + 21 ** 3)
    fine = [c for c in configs if c.cells.initial_count == 200 and c.oxygen.grid.dx_um == 10.0][0]
    assert sw.run_cost(fine) == 2.0 * (200 + 41 ** 3)


@pytest.mark.parametrize("batched", [False, True])
def test_two_gloo_ranks_run_disjoint_shares_and_gather_the_summary(tmp_path, monkeypatch, batched):
    world = 2
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    out_dir = str(tmp_path / "sharded")
    ran_dir = str(tmp_path)
    procs = [ctx.Process(target=_worker, args=(r, world, port, out_dir, batched, ran_dir, queue)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(queue.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0

    spec = _spec()
    sweep = sw.Sweep(spec, BASE)
    labels = [label for label, _, _ in sweep.configs]
    parts = sw.partition_runs([sw.run_cost(c) for _, _, c in sweep.configs], world)
    for rank in range(world):
        ran = open(os.path.join(ran_dir, f"rank{rank}.txt")).read().split()
        assert sorted(ran) == sorted(labels[i] for i in parts[rank])  # each rank ran exactly its share
    assert _same_rows(got[0], got[1])  # every rank returns the whole summary

    # the one-process sweep with the same executor gives the same rows, in the same order
    monkeypatch.setattr(sw, "_run_experiment", _fake_experiment)
    monkeypatch.setattr(sw, "run_batched", _fake_batched)
    monkeypatch.delenv("WBC_TEST_RAN", raising=False)
    single = sweep.run(str(tmp_path / "single"), batched=batched, rank=0, world=1)
    assert _same_rows(got[0], single, skip=("run_dir",))
    assert [row["label"] for row in got[0]] == labels

    with open(os.path.join(out_dir, "summary.csv"), newline="") as f:
        written = list(csv.DictReader(f))
    assert [r["label"] for r in written] == labels
    assert [int(float(r["final_cells"])) for r in written] == [int(row["final_cells"]) for row in single]


def _is_failing(config) -> bool:
    return config.cells.initial_count == 3000 and config.oxygen.grid.dx_um == 10.0 and config.simulation.seed == 0


def _failing_experiment(config, run_dir, device):
    # one run (3000 cells, 10 um spacing, seed 0) fails, as a run that ran out of device memory would
    if _is_failing(config):
        raise RuntimeError("simulated failure of one run")
    return _fake_experiment(config, run_dir, device)


def _failing_worker(rank, world, port, out_dir, ran_dir, queue):
    import torch.distributed as dist
    from datetime import timedelta

    os.environ["WBC_TEST_RAN"] = os.path.join(ran_dir, f"rank{rank}.txt")
    sw._run_experiment = _failing_experiment
    # a short collective timeout: a rank left waiting in the gather would fail the test by time
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world,
                            timeout=timedelta(seconds=60))
    try:
        sw.Sweep(_spec(), BASE).run(out_dir, batched=False)
        queue.put((rank, "no error"))
    except sw.SweepRankError as exc:
        queue.put((rank, f"SweepRankError: {exc}"))
    except Exception as exc:  # noqa: BLE001
        queue.put((rank, f"{type(exc).__name__}: {exc}"))
    finally:
        dist.destroy_process_group()


def test_a_failing_run_on_one_rank_raises_on_every_rank_without_a_hang(tmp_path):
    world = 2
    spec = _spec()
    sweep = sw.Sweep(spec, BASE)
    parts = sw.partition_runs([sw.run_cost(c) for _, _, c in sweep.configs], world)
    failing = [r for r in range(world) for i in parts[r] if _is_failing(sweep.configs[i][2])]
    assert len(failing) == 1  # one rank's share holds the failing run; the other rank's runs all succeed
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_failing_worker, args=(r, world, port, str(tmp_path / "sweep"), str(tmp_path), queue))
             for r in range(world)]
    for p in procs:
        p.start()
    got = dict(queue.get(timeout=50) for _ in range(world))  # well inside the 60 s collective timeout
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in range(world):
        assert got[rank].startswith("SweepRankError"), got[rank]
        assert f"rank {failing[0]}" in got[rank] and "simulated failure of one run" in got[rank]

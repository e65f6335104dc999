"""Parameter sweeps: a base configuration, a grid of overrides and a list of seeds
(reference: simulation/sweep.py).

Sweep file (YAML)::

    name: oxygen_boundary
    seeds: [0, 1, 2]
    overrides:                       # applied to every run
      simulation.duration_h: 288
    grid:                            # cartesian product, one run per combination and seed
      oxygen.boundary_mmHg: [20, 38, 60, 100, 150]

Every run is an ordinary run directory under the sweep's directory, and ``summary.csv`` collects,
per run, the swept values, the seed, the status, onset times and radii of hypoxia and necrosis,
and the final metrics row.

``Sweep.run(..., batched=True)`` advances every run of the sweep together on one GPU
(:class:`simulation.batch.SpheroidBatch`: one launch per stage for all members, one persistent
launch for all field solves) when every run is a plain oxygen run (no extra species, network or
tissue region) with the same solver settings and time steps; each member's states are
bit-identical to its run alone. Otherwise the runs go one after another as in the reference.

Under ``torch.distributed`` (one process per GPU, e.g. ``torchrun``) the runs are independent, so
the sweep is sharded by run: :func:`partition_runs` gives each rank a share balanced on the
estimated work of :func:`run_cost` (cell-steps plus node-steps), each rank runs its share (batched
where possible) into the same sweep directory, and rank 0 gathers the summary rows, which are the
only data that crosses ranks, and writes ``summary.csv`` and ``metadata.json`` in sweep order.
"""

from __future__ import annotations

import copy
import csv
import dataclasses
import datetime as dt
import itertools
import json
import math
import shutil
import time
from dataclasses import dataclass, field
from pathlib import Path
from typing import Callable

import torch

from warpbiocell_gb300.io.run_output import METRIC_COLUMNS, RunOutput
from warpbiocell_gb300.metrics.timeseries import onset_summary
from warpbiocell_gb300.simulation import yaml_subset
from warpbiocell_gb300.simulation.config import ConfigError, apply_overrides, config_from_dict, read_yaml
from warpbiocell_gb300.simulation.experiment import Experiment, RunResult

ONSET_COLUMNS = ["hypoxia_onset_time_h", "hypoxia_onset_radius_um", "necrosis_onset_time_h",
                 "necrosis_onset_radius_um"]


@dataclass(frozen=True)
class SweepSpec:
    name: str
    seeds: tuple[int, ...] = (0,)
    overrides: dict = field(default_factory=dict)  # dotted key -> value
    grid: dict = field(default_factory=dict)  # dotted key -> list of values

    def __post_init__(self):
        if not self.name:
            raise ConfigError("sweep needs a name")
        if not self.seeds:
            raise ConfigError("sweep needs at least one seed")
        for key, values in self.grid.items():
            if not isinstance(values, (list, tuple)) or not values:
                raise ConfigError(f"grid.{key} must be a non-empty list")

    @property
    def grid_keys(self) -> list[str]:
        return list(self.grid)

    def runs(self) -> list[tuple[str, dict]]:
        """``(label, {dotted key: value})`` for every grid combination and seed, in order."""
        out = []
        combos = itertools.product(*(self.grid[k] for k in self.grid_keys)) if self.grid else [()]
        for combo in combos:
            values = dict(zip(self.grid_keys, combo))
            for seed in self.seeds:
                parts = [f"{k.split('.')[-1]}={_fmt(v)}" for k, v in values.items()] + [f"seed={seed}"]
                out.append(("_".join(parts), {**values, "simulation.seed": seed}))
        return out


def _fmt(value) -> str:
    return f"{value:g}" if isinstance(value, (int, float)) and not isinstance(value, bool) else str(value)


def load_sweep(path: str | Path) -> SweepSpec:
    data = read_yaml(path)
    unknown = set(data) - {"name", "seeds", "overrides", "grid"}
    if unknown:
        raise ConfigError(f"sweep: unknown keys {sorted(unknown)}")
    return SweepSpec(name=str(data.get("name", Path(path).stem)), seeds=tuple(int(s) for s in data.get("seeds", [0])),
                     overrides=dict(data.get("overrides") or {}), grid=dict(data.get("grid") or {}))


def _yaml(value) -> str:
    return yaml_subset.safe_dump(value, default_flow_style=True).strip().removesuffix("\n...")


def build_run_config(base: dict, spec: SweepSpec, label: str, values: dict):
    data = copy.deepcopy(base)
    apply_overrides(data, [f"{k}={_yaml(v)}" for k, v in spec.overrides.items()])
    apply_overrides(data, [f"{k}={_yaml(v)}" for k, v in values.items()])
    data["name"] = label
    return config_from_dict(data)


def batchable(configs) -> bool:
    """Plain oxygen runs with one set of solver settings and time steps, no region or network."""
    first = configs[0]
    for c in configs:
        if not c.oxygen.enabled or c.species or c.oxygen.uptake_state_factors or c.geometry.enabled \
                or c.network.enabled or c.lifecycle.phenotype_model != "rules":
            return False
        if c.oxygen.solver != first.oxygen.solver or c.simulation.dt_cells_h != first.simulation.dt_cells_h \
                or c.simulation.dt_mechanics_h != first.simulation.dt_mechanics_h \
                or c.simulation.duration_h != first.simulation.duration_h:
            return False
    return True


def run_cost(config) -> float:
    """Estimated work of one run: cell-steps of its initial population plus node-steps of its
    field grids (a node update per sweep costs about a thousandth of a cell-step and warm solves
    take hundreds of sweeps, so one node-step weighs about one cell-step)."""
    steps = max(1, int(round(config.simulation.duration_h / config.simulation.dt_cells_h)))
    nodes = 0
    if config.oxygen.enabled:
        n = int(math.ceil(config.oxygen.grid.box_um / config.oxygen.grid.dx_um)) + 1
        nodes = n ** 3 * (1 + len(config.species))
    return float(steps) * float(config.cells.initial_count + nodes)


class SweepRankError(RuntimeError):
    """A sharded sweep in which at least one rank's runs raised; raised on every rank, after the
    ranks have exchanged what happened, with each failing rank's runs and error."""


def partition_runs(costs: list[float], world: int) -> list[list[int]]:
    """Run indices per rank: longest run first onto the least loaded rank (lowest rank on ties),
    each share in sweep order. Deterministic, so every rank computes the same partition."""
    if world < 1:
        raise ValueError("world must be >= 1")
    loads = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(world), key=lambda r: (loads[r], r))
        parts[r].append(i)
        loads[r] += costs[i]
    return [sorted(p) for p in parts]


def _rank_world(rank: int | None, world: int | None) -> tuple[int, int]:
    if rank is not None and world is not None:
        return rank, world
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def _run_experiment(config, run_dir: Path, device):
    return Experiment(config, device=device).run(run_dir, log=None)


class Sweep:
    def __init__(self, spec: SweepSpec, base: dict, base_path: Path | None = None, sweep_path: Path | None = None):
        self.spec = spec
        self.base = base
        self.base_path = base_path
        self.sweep_path = sweep_path
        self.configs = [(label, values, build_run_config(base, spec, label, values)) for label, values in spec.runs()]
        for _, _, config in self.configs:
            config.validate()

    def run(self, out_dir: str | Path, device: str | None = None, figures: bool = False,
            log: Callable[[str], None] | None = None, batched: bool = False, rank: int | None = None,
            world: int | None = None) -> list[dict]:
        """Run every configuration and return the summary rows in sweep order. ``rank``/``world``
        default to the initialised ``torch.distributed`` group (else one process); with
        ``world > 1`` this process runs its share of the runs, see :func:`partition_runs`."""
        rank, world = _rank_world(rank, world)
        if world > 1:
            return self._run_sharded(Path(out_dir), device, figures, log, batched, rank, world)
        out_dir = Path(out_dir)
        out_dir.mkdir(parents=True, exist_ok=True)
        if self.sweep_path is not None:
            shutil.copyfile(self.sweep_path, out_dir / "sweep.yaml")
        if self.base_path is not None:
            shutil.copyfile(self.base_path, out_dir / "base_config.yaml")
        metadata = {"name": self.spec.name, "started": dt.datetime.now(dt.timezone.utc).isoformat(),
                    "finished": None, "spec": dataclasses.asdict(self.spec), "runs": []}
        configs = []
        for label, values, config in self.configs:
            if not figures:
                config = dataclasses.replace(config, output=dataclasses.replace(config.output, figures=False))
            configs.append((label, values, config))
        use_batch = batched and batchable([c for _, _, c in configs])
        metadata["batched"] = use_batch
        if batched and not use_batch and log:
            log("runs differ in species, network, region, solver settings or time steps: running them one by one")
        columns = ["label", "run_dir", "seed", *self.spec.grid_keys, "status", "wall_s", *ONSET_COLUMNS,
                   *[f"final_{c}" for c in METRIC_COLUMNS]]
        rows = []
        with (out_dir / "summary.csv").open("w", newline="") as f:
            writer = csv.DictWriter(f, fieldnames=columns)
            writer.writeheader()

            def finish(label, values, config, result, run_dir):
                row = self._row(label, values, config, result, run_dir)
                rows.append(row)
                writer.writerow(row)
                f.flush()
                metadata["runs"].append({"label": label, "status": result.status, "wall_s": result.wall_s})
                (out_dir / "metadata.json").write_text(json.dumps(metadata, indent=2, default=str))
                if log:
                    log(f"    {label}: {result.status}  cells={result.metrics[-1]['cells']}  "
                        f"R={result.metrics[-1]['spheroid_radius_um']:.0f} um  wall={result.wall_s:.0f} s")

            if use_batch:
                results = run_batched([c for _, _, c in configs], [out_dir / label for label, _, _ in configs],
                                      device=device, log=log)
                for (label, values, config), result in zip(configs, results):
                    finish(label, values, config, result, out_dir / label)
            else:
                for index, (label, values, config) in enumerate(configs, start=1):
                    if log:
                        log(f"[{index}/{len(configs)}] {label}")
                    result = _run_experiment(config, out_dir / label, device)
                    finish(label, values, config, result, out_dir / label)
        metadata["finished"] = dt.datetime.now(dt.timezone.utc).isoformat()
        (out_dir / "metadata.json").write_text(json.dumps(metadata, indent=2, default=str))
        return rows

    def _row(self, label, values, config, result, run_dir) -> dict:
        return {"label": label, "run_dir": str(run_dir), "seed": config.simulation.seed,
                **{k: values[k] for k in self.spec.grid_keys}, "status": result.status, "wall_s": result.wall_s,
                **onset_summary(result.metrics), **{f"final_{k}": v for k, v in result.metrics[-1].items()}}

    def _run_sharded(self, out_dir: Path, device, figures, log, batched, rank: int, world: int) -> list[dict]:
        import os

        import torch.distributed as dist

        if device is None and torch.cuda.is_available():
            device = f"cuda:{int(os.environ.get('LOCAL_RANK', rank)) % torch.cuda.device_count()}"
        out_dir.mkdir(parents=True, exist_ok=True)
        started = dt.datetime.now(dt.timezone.utc).isoformat()
        configs = []
        for label, values, config in self.configs:
            if not figures:
                config = dataclasses.replace(config, output=dataclasses.replace(config.output, figures=False))
            configs.append((label, values, config))
        use_batch = batched and batchable([c for _, _, c in configs])
        mine = partition_runs([run_cost(c) for _, _, c in configs], world)[rank]
        done: list[tuple[int, dict]] = []
        failure: dict | None = None
        # Whatever happens to this rank's runs, it still takes part in the gather below: a rank
        # that raised before it would leave every other rank blocked in the collective until the
        # process group times out. Its error travels in the gathered data instead and every rank
        # raises it after the gather.
        try:
            if mine:
                if use_batch:
                    results = run_batched([configs[i][2] for i in mine], [out_dir / configs[i][0] for i in mine],
                                          device=device, log=log)
                else:
                    results = [_run_experiment(configs[i][2], out_dir / configs[i][0], device) for i in mine]
                for i, result in zip(mine, results):
                    label, values, config = configs[i]
                    done.append((i, self._row(label, values, config, result, out_dir / label)))
                    if log:
                        log(f"    [rank {rank}] {label}: {result.status}  cells={result.metrics[-1]['cells']}")
        except Exception as exc:  # noqa: BLE001 - re-raised on every rank after the gather
            failure = {"rank": rank, "runs": [configs[i][0] for i in mine if i not in {j for j, _ in done}],
                       "error": f"{type(exc).__name__}: {exc}"}
            local_exc: Exception | None = exc
        else:
            local_exc = None
        gathered: list = [None] * world
        dist.all_gather_object(gathered, {"rows": done, "failure": failure})
        failures = [part["failure"] for part in gathered if part["failure"] is not None]
        if failures:
            what = "; ".join(f"rank {f['rank']} ({', '.join(f['runs']) or 'no run'}): {f['error']}" for f in failures)
            if local_exc is not None:
                raise SweepRankError(f"sweep failed on {len(failures)} of {world} ranks: {what}") from local_exc
            raise SweepRankError(f"sweep failed on {len(failures)} of {world} ranks: {what}")
        rows = [row for _, row in sorted((item for part in gathered for item in part["rows"]), key=lambda t: t[0])]
        if rank == 0:
            if self.sweep_path is not None:
                shutil.copyfile(self.sweep_path, out_dir / "sweep.yaml")
            if self.base_path is not None:
                shutil.copyfile(self.base_path, out_dir / "base_config.yaml")
            columns = ["label", "run_dir", "seed", *self.spec.grid_keys, "status", "wall_s", *ONSET_COLUMNS,
                       *[f"final_{c}" for c in METRIC_COLUMNS]]
            with (out_dir / "summary.csv").open("w", newline="") as f:
                writer = csv.DictWriter(f, fieldnames=columns)
                writer.writeheader()
                for row in rows:
                    writer.writerow(row)
            metadata = {"name": self.spec.name, "started": started,
                        "finished": dt.datetime.now(dt.timezone.utc).isoformat(),
                        "spec": dataclasses.asdict(self.spec), "batched": use_batch, "world": world,
                        "runs": [{"label": r["label"], "status": r["status"], "wall_s": r["wall_s"]} for r in rows]}
            (out_dir / "metadata.json").write_text(json.dumps(metadata, indent=2, default=str))
        return rows


def run_batched(configs, run_dirs=None, device=None, log: Callable[[str], None] | None = None) -> list[RunResult]:
    """Run plain-oxygen configurations together as one :class:`SpheroidBatch` (see :func:`batchable`).

    Records the same metrics, profiles and checkpoints as :meth:`Experiment.run` at the same
    steps. A member whose daughters would exceed its capacity stops there with status
    ``capacity_exceeded``: its lifecycle decisions of that step stand and no daughter is placed,
    as in a plain run, but the batch still applies that step's contact substeps to it before the
    final row is recorded.
    """
    from warpbiocell_gb300.simulation.batch import BatchMember, SpheroidBatch

    if not batchable(configs):
        raise ValueError("the configurations cannot be batched")
    exps = [Experiment(c, device=device) for c in configs]
    outputs = []
    for k, (exp, cfg) in enumerate(zip(exps, configs)):
        out = None
        if run_dirs is not None:
            out = RunOutput(Path(run_dirs[k]), None, cfg.to_dict(), exp.device, cfg.simulation.seed)
            out.metadata["warnings"] = list(exp.warnings)
            out.metadata["batched_with"] = len(configs)
            out.write_metadata()
        outputs.append(out)
    from warpbiocell_gb300.cells.mechanics import contact_substep

    for exp in exps:
        contact_substep(exp.population, exp.grid, exp.contact, dt=0.0)
        exp.oxygen.update(exp.population)
    stepping = exps[0].stepping
    batch = SpheroidBatch([BatchMember(e.population, e.grid, e.oxygen, e.lifecycle, e.contact) for e in exps],
                          stepping)
    out_cfg = configs[0].output

    def every(hours):
        return max(1, int(round(hours / stepping.dt_cells)))

    metrics_every, profile_every, checkpoint_every = (every(out_cfg.metrics_every_h), every(out_cfg.profile_every_h),
                                                      every(out_cfg.checkpoint_every_h))
    results = [RunResult(status="completed", output_dir=Path(d) if run_dirs is not None else None)
               for d in (run_dirs or [None] * len(exps))]
    active = [True] * len(exps)
    t_start = time.perf_counter()

    def record(k, wall, sweeps, due=(True, True, True)):
        exp, result, out = exps[k], results[k], outputs[k]
        row, prof = exp.observe(wall, sweeps)
        if due[0]:
            result.metrics.append(row)
            if out:
                out.write_metrics(row)
        if due[1]:
            result.profiles.append((exp.time_h, prof))
            if out:
                out.write_profile(exp.time_h, prof)
        if due[2] and out:
            exp.save(out.checkpoint_path(exp.time_h))

    for k in range(len(exps)):
        record(k, 0.0, 0)
    n_steps = configs[0].n_steps
    # The solve plan is re-made once from the mean sweep counts of steps 2-4 (the first step's
    # solve starts from the initial steady state and is short); until then steps run uncaptured.
    plan_after, history = 4, []
    for step in range(1, n_steps + 1):
        batch.step()
        if step <= plan_after:
            if step > 1:
                history.append([r.sweeps for r in batch.reports()])
            if step == plan_after:
                batch.rebalance([sum(col) / len(col) for col in zip(*history)])
                batch.capture()
        last = step == n_steps
        due = (step % metrics_every == 0 or last, step % profile_every == 0 or last,
               step % checkpoint_every == 0 or last)
        status = batch.status_codes()
        failed = [k for k in range(len(exps)) if active[k] and status[k] != 0]
        if any(due) or failed:
            batch.sync()
            torch.cuda.synchronize(exps[0].device)
            wall = time.perf_counter() - t_start
            reports = batch.reports()
            for k, exp in enumerate(exps):
                if not active[k]:
                    continue
                exp.time_h = step * stepping.dt_cells if k not in failed else (step - 1) * stepping.dt_cells
                if k in failed:
                    results[k].status = "capacity_exceeded"
                    record(k, wall, reports[k].sweeps)
                    active[k] = False
                    if log:
                        log(f"{configs[k].name}: stopping at t={exp.time_h:.2f} h (capacity)")
                elif any(due):
                    record(k, wall, reports[k].sweeps, due)
        if not any(active):
            break
    torch.cuda.synchronize(exps[0].device)
    wall = time.perf_counter() - t_start
    for k, (exp, result, out) in enumerate(zip(exps, results, outputs)):
        result.wall_s = wall
        result.summary = {**result.metrics[-1], "steps": int(round(exp.time_h / stepping.dt_cells)),
                          "status": result.status}
        if out:
            out.finish(result.status, wall, result.summary)
    return results

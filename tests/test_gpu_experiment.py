"""The experiment runner, checkpoints and sweeps on the device (reference: tests/test_experiment.py,
tests/test_sweep.py): a run writes its directory, a run resumed from one of its checkpoints ends
bit-identical to the uninterrupted run, and a batched sweep reports exactly the rows of the same
runs made one by one."""

import csv
import json

import numpy as np
import pytest

from warpbiocell_gb300.io.checkpoints import load_checkpoint
from warpbiocell_gb300.simulation.config import config_from_dict
from warpbiocell_gb300.simulation.experiment import Experiment
from warpbiocell_gb300.simulation.sweep import Sweep, SweepSpec

pytestmark = pytest.mark.gpu


def _base(**over):
    data = {
        "name": "small",
        "simulation": {"duration_h": 2.0, "dt_cells_h": 0.5, "dt_mechanics_h": 0.05, "seed": 3, "device": "cuda:0"},
        "cells": {"initial_count": 300, "max_cells": 4000, "radius_um": 8.0},
        "mechanics": {"stiffness": 10.0, "damping": 1.0, "margin_um": 2.0},
        "lifecycle": {"division_rate_per_h": 0.3, "hypoxia_threshold_mmHg": 20.0, "death_threshold_mmHg": 2.0},
        "oxygen": {"boundary_mmHg": 38.0, "uptake_max_mmHg_um3_per_h": 1.0e9, "grid": {"box_um": 400.0, "dx_um": 20.0}},
        "output": {"metrics_every_h": 0.5, "profile_every_h": 1.0, "checkpoint_every_h": 1.0, "figures": False},
    }
    for key, value in over.items():
        section, name = key.split("__")
        data[section][name] = value
    return data


def _strip(row):
    """A row without its wall time, NaN made comparable."""
    return {k: ("nan" if isinstance(v, float) and v != v else v) for k, v in row.items() if k != "wall_s"}


def test_experiment_run_writes_the_run_directory(tmp_path):
    cfg = config_from_dict(_base())
    result = Experiment(cfg).run(tmp_path / "run")
    assert result.status == "completed"
    assert [r["time_h"] for r in result.metrics] == [0.0, 0.5, 1.0, 1.5, 2.0]
    assert result.metrics[-1]["cells"] > 300 and result.summary["steps"] == 4
    assert result.metrics[-1]["hypoxic_cells"] > 0
    with open(tmp_path / "run" / "metrics.csv") as f:
        rows = list(csv.DictReader(f))
    assert len(rows) == 5 and int(rows[-1]["cells"]) == result.metrics[-1]["cells"]
    meta = json.loads((tmp_path / "run" / "metadata.json").read_text())
    assert meta["status"] == "completed" and meta["summary"]["cells"] == result.metrics[-1]["cells"]
    ckpts = sorted((tmp_path / "run" / "checkpoint").glob("*.npz"))
    assert [p.name for p in ckpts] == ["state_0000.00h.npz", "state_0001.00h.npz", "state_0002.00h.npz"]
    data = load_checkpoint(ckpts[-1])
    assert int(data["count"]) == result.metrics[-1]["cells"] and data["rng_state"].dtype == np.uint32
    assert (tmp_path / "run" / "config.yaml").exists() and (tmp_path / "run" / "profiles.csv").exists()


def test_resume_from_checkpoint_is_bit_identical(tmp_path):
    cfg = config_from_dict(_base())
    full = Experiment(cfg)
    res_full = full.run(tmp_path / "full")
    resumed = Experiment(cfg)
    resumed.resume(tmp_path / "full" / "checkpoint" / "state_0001.00h.npz")
    assert resumed.time_h == 1.0
    res = resumed.run(tmp_path / "resumed")
    n = full.population.count
    assert resumed.population.count == n
    np.testing.assert_array_equal(resumed.population.positions_numpy(), full.population.positions_numpy())
    np.testing.assert_array_equal(resumed.population.states_numpy(), full.population.states_numpy())
    np.testing.assert_array_equal(resumed.population.rng_numpy(), full.population.rng_numpy())
    np.testing.assert_array_equal(resumed.oxygen.numpy(), full.oxygen.numpy())
    assert [_strip(r) for r in res.metrics[1:]] == [_strip(r) for r in res_full.metrics[3:]]


def test_batched_sweep_reports_the_rows_of_sequential_runs(tmp_path):
    spec = SweepSpec(name="o2", seeds=(0, 1), grid={"oxygen.boundary_mmHg": [30.0, 60.0]})
    base = _base()
    seq = Sweep(spec, base).run(tmp_path / "seq")
    bat = Sweep(spec, base).run(tmp_path / "bat", batched=True)
    meta = json.loads((tmp_path / "bat" / "metadata.json").read_text())
    assert meta["batched"] is True
    assert len(seq) == len(bat) == 4
    for a, b in zip(seq, bat):
        assert a["label"] == b["label"] and a["status"] == b["status"] == "completed"
        fa = _strip({k: v for k, v in a.items() if k.startswith("final_") and k != "final_wall_s"})
        fb = _strip({k: v for k, v in b.items() if k.startswith("final_") and k != "final_wall_s"})
        assert fa == fb
    with open(tmp_path / "bat" / seq[1]["label"] / "metrics.csv") as f:
        rows_b = [_strip(r) for r in csv.DictReader(f)]
    with open(tmp_path / "seq" / seq[1]["label"] / "metrics.csv") as f:
        rows_a = [_strip(r) for r in csv.DictReader(f)]
    assert rows_a == rows_b


def test_capacity_stop_is_reported():
    cfg = config_from_dict(_base(cells__max_cells=320, lifecycle__division_rate_per_h=2.0))
    result = Experiment(cfg).run()
    assert result.status == "capacity_exceeded"
    assert result.metrics[-1]["cells"] <= 320


def test_on_metrics_observer_receives_every_row():
    """Reference tests/test_experiment.py: the observer sees every metrics row as it is made."""
    rows = []
    result = Experiment(config_from_dict(_base())).run(on_metrics=rows.append)
    assert [r["time_h"] for r in rows] == [r["time_h"] for r in result.metrics] == [0.0, 0.5, 1.0, 1.5, 2.0]
    assert rows[-1]["cells"] == result.summary["cells"]


def test_in_memory_runs_are_reproducible_and_seed_dependent():
    a = Experiment(config_from_dict(_base())).run()
    b = Experiment(config_from_dict(_base())).run()
    c = Experiment(config_from_dict(_base(simulation__seed=4))).run()
    for key in ("cells", "dead_cells", "spheroid_radius_um", "oxygen_cells_min_mmHg"):
        np.testing.assert_array_equal(a.metric(key), b.metric(key))
    assert a.summary["cells"] != c.summary["cells"] or a.summary["spheroid_radius_um"] != c.summary["spheroid_radius_um"]


def test_oxygen_can_be_disabled(tmp_path):
    result = Experiment(config_from_dict(_base(oxygen__enabled=False))).run(tmp_path / "run")
    assert result.status == "completed"
    assert result.summary["hypoxic_cells"] == 0
    assert np.isnan(result.summary["oxygen_cells_min_mmHg"])
    assert (tmp_path / "run" / "metrics.csv").exists()


def test_experiment_in_a_tissue_region_from_a_mask_file(tmp_path):
    # reference: simulation/experiment.py:141-145 (geometry.shape = mask, a NIfTI label image)
    from tests.test_masks import _voxel_sphere, _write_single

    mask, origin, _ = _voxel_sphere(n=30, voxel=20.0, radius=120.0)
    _write_single(tmp_path / "lesion.nii.gz", np.where(mask, 2, 0).astype(np.int16), (0.02, 0.02, 0.02),
                  compress=True)
    data = _base(simulation__duration_h=1.0, cells__max_cells=6000)
    data["geometry"] = {"enabled": True, "shape": "mask", "mask_file": str(tmp_path / "lesion.nii.gz"),
                        "mask_label": 2, "mask_origin_um": [float(origin)] * 3, "seed_fill": True}
    exp = Experiment(config_from_dict(data))
    assert exp.region.name == "lesion.nii.gz" and exp.population.count > 500
    result = exp.run()
    assert result.status == "completed"
    assert all(row["cells_outside_tissue"] == 0 for row in result.metrics)

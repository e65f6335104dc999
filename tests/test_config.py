"""Experiment configuration, the YAML subset reader and sweep specifications (reference:
tests/test_config.py, tests/test_sweep.py): host logic only, no device."""

import math
import os
from pathlib import Path

import numpy as np
import pytest

from warpbiocell_gb300.simulation import yaml_subset
from warpbiocell_gb300.simulation.config import (ConfigError, ExperimentConfig, apply_overrides, config_from_dict,
                                                 load_config)
from warpbiocell_gb300.simulation.sweep import SweepSpec, batchable, build_run_config, load_sweep
from warpbiocell_gb300.metrics.timeseries import onset, onset_summary

CONFIG_TEXT = """\
name: small_spheroid   # provenance comments travel with the file
simulation:
  duration_h: 2.0
  dt_cells_h: 0.5
  dt_mechanics_h: 0.05
  seed: 3
cells:
  initial_count: 200
  max_cells: 5000
  radius_um: 8.0
mechanics:
  stiffness: 10.0
  damping: 1.0
  margin_um: 2.0
lifecycle:
  division_rate_per_h: 0.2
  hypoxia_threshold_mmHg: 8.0
oxygen:
  diffusion_um2_per_h: 7.2e6     # YAML 1.1 reads this as a string; the loader converts it
  uptake_state_factors: {hypoxic: 0.5}
  grid:
    box_um: 400.0
    dx_um: 20.0
  solver: {omega: 1.8, tolerance: 1.0e-5, max_sweeps: 2000, check_every: 10}
species:
  - name: glucose
    unit: mM
    diffusion_um2_per_h: 2.16e6
    uptake_max_by_state: {proliferative: 1.2e4, quiescent: 1.2e4, hypoxic: 1.2e4}
  - name: lactate
    production_by_state: {hypoxic: 2.4e4}
    production_source: glucose
output:
  metrics_every_h: 0.5
  figures: false
"""


def test_yaml_subset_reads_block_and_flow_collections():
    data = yaml_subset.safe_load(CONFIG_TEXT)
    assert data["name"] == "small_spheroid"
    assert data["simulation"] == {"duration_h": 2.0, "dt_cells_h": 0.5, "dt_mechanics_h": 0.05, "seed": 3}
    assert float(data["oxygen"]["diffusion_um2_per_h"]) == 7.2e6
    assert data["oxygen"]["uptake_state_factors"] == {"hypoxic": 0.5}
    assert data["oxygen"]["solver"]["max_sweeps"] == 2000
    assert [s["name"] for s in data["species"]] == ["glucose", "lactate"]
    assert data["species"][1]["production_source"] == "glucose"
    assert data["output"]["figures"] is False
    assert yaml_subset.scalar("[20, 38, 60]") == [20, 38, 60]
    assert yaml_subset.scalar("null") is None and yaml_subset.scalar("'a: b'") == "a: b"
    text = yaml_subset.safe_dump({"a": {"b": [1, 2], "c": "x y"}, "d": [{"e": 1}], "f": None})
    assert yaml_subset.safe_load(text) == {"a": {"b": [1, 2], "c": "x y"}, "d": [{"e": 1}], "f": None}


def test_load_config_builds_parameter_objects(tmp_path):
    path = tmp_path / "c.yaml"
    path.write_text(CONFIG_TEXT)
    cfg = load_config(path, overrides=["oxygen.boundary_mmHg=60", "cells.max_cells=6000"])
    assert cfg.oxygen.boundary_mmHg == 60.0 and cfg.cells.max_cells == 6000
    assert cfg.oxygen.diffusion_um2_per_h == 7.2e6 and cfg.n_steps == 4
    assert cfg.has_glucose
    st = cfg.stepping()
    assert st.mechanics_substeps == 10
    contact = cfg.contact_params()
    assert contact.query_radius == 2 * 8.0 + 2.0 and contact.rate == 10.0
    lc = cfg.lifecycle_params()
    assert lc.division_rate == 0.2 and lc.glucose_threshold == 0.0
    species = cfg.species_params()
    assert [s.name for s in species] == ["glucose", "lactate"] and species[1].production_source == "glucose"
    assert cfg.grid_geometry().shape == (21, 21, 21)
    assert cfg.solver_settings().check_every == 10
    warnings = cfg.validate()
    assert isinstance(warnings, list)
    assert config_from_dict(cfg.to_dict()) == cfg  # round trip through plain dicts


def test_config_errors():
    with pytest.raises(ConfigError, match="unknown keys"):
        config_from_dict({"cells": {"max_cell": 10}})
    with pytest.raises(ConfigError, match="expected an integer"):
        config_from_dict({"cells": {"max_cells": 1.5}})
    with pytest.raises(ConfigError, match="expected true/false"):
        config_from_dict({"output": {"figures": "yes please"}})
    with pytest.raises(ConfigError, match="does not fit"):
        config_from_dict({"cells": {"initial_count": 100000, "max_cells": 200000}}).validate()
    with pytest.raises(ConfigError, match="unique"):
        config_from_dict({"species": [{"name": "glucose"}, {"name": "glucose"}]}).validate()
    with pytest.raises(ConfigError, match="earlier species"):
        config_from_dict({"species": [{"name": "lactate", "production_source": "glucose"}]}).validate()
    with pytest.raises(ConfigError, match="network.enabled"):
        config_from_dict({"lifecycle": {"phenotype_model": "network"}}).validate()
    with pytest.raises(ValueError, match="rate\\*dt"):
        config_from_dict({"mechanics": {"stiffness": 100.0}, "simulation": {"dt_mechanics_h": 0.025}}).validate()
    with pytest.raises(ConfigError, match="section.key=value"):
        apply_overrides({}, ["no_equals_sign"])
    warnings = config_from_dict({"lifecycle": {"division_rate_per_h": 1.0}, "cells": {"max_cells": 2000}}).validate()
    assert any("exponential growth" in w for w in warnings)


def test_geometry_config_validation():
    cfg = config_from_dict({"geometry": {"enabled": True, "shape": "ellipsoid", "radii_um": [120.0, 90.0, 60.0]},
                            "cells": {"max_cells": 5000}, "oxygen": {"grid": {"box_um": 400.0}}})
    cfg.validate()
    assert cfg.tissue_shape().bounds[1][0] == 120.0
    with pytest.raises(ConfigError, match="one-voxel margin"):
        config_from_dict({"geometry": {"enabled": True, "shape": "sphere", "radii_um": [395.0]}}).validate()
    with pytest.raises(ConfigError, match="sphere, ellipsoid"):
        config_from_dict({"geometry": {"enabled": True, "shape": "cube"}}).validate()


def test_sweep_spec_runs_labels_and_configs(tmp_path):
    spec_path = tmp_path / "s.yaml"
    spec_path.write_text("name: o2\nseeds: [0, 1]\noverrides:\n  simulation.duration_h: 1.0\n"
                         "grid:\n  oxygen.boundary_mmHg: [20, 38.5]\n")
    spec = load_sweep(spec_path)
    runs = spec.runs()
    assert [label for label, _ in runs] == ["boundary_mmHg=20_seed=0", "boundary_mmHg=20_seed=1",
                                            "boundary_mmHg=38.5_seed=0", "boundary_mmHg=38.5_seed=1"]
    base = yaml_subset.safe_load(CONFIG_TEXT)
    base.pop("species")
    base["oxygen"].pop("uptake_state_factors")
    configs = [build_run_config(base, spec, label, values) for label, values in runs]
    assert configs[2].oxygen.boundary_mmHg == 38.5 and configs[1].simulation.seed == 1
    assert configs[0].simulation.duration_h == 1.0 and configs[3].name == "boundary_mmHg=38.5_seed=1"
    assert batchable(configs)
    assert not batchable([config_from_dict(yaml_subset.safe_load(CONFIG_TEXT))])
    with pytest.raises(ConfigError):
        SweepSpec(name="x", grid={"oxygen.boundary_mmHg": []})
    with pytest.raises(ConfigError):
        SweepSpec(name="")


def test_onsets():
    rows = [{"time_h": 0.0, "hypoxic_cells": 0, "dead_cells": 0, "spheroid_radius_um": 50.0},
            {"time_h": 1.0, "hypoxic_cells": 3, "dead_cells": 0, "spheroid_radius_um": 60.0},
            {"time_h": 2.0, "hypoxic_cells": 5, "dead_cells": 1, "spheroid_radius_um": 70.0}]
    assert onset(rows, "hypoxic_cells") == (1.0, 60.0)
    s = onset_summary(rows)
    assert s["necrosis_onset_time_h"] == 2.0 and s["necrosis_onset_radius_um"] == 70.0
    assert all(math.isnan(v) for v in onset(rows[:1], "dead_cells"))


def test_default_config_matches_documented_defaults():
    cfg = ExperimentConfig()
    assert cfg.oxygen.boundary_mmHg == 38.0 and cfg.oxygen.solver.max_sweeps == 2000
    assert np.isclose(cfg.lifecycle.division_rate_per_h, 0.0289)
    assert cfg.mechanics.wall_rate_per_h == 10.0 and cfg.output.shell_width_um == 20.0



def test_config_errors_name_the_offending_key():
    # reference: tests/test_config.py:30-41 (unknown keys and type errors carry their dotted path)
    with pytest.raises(ConfigError, match=r"config\.oxygen: unknown keys \['boundary_mmhg'\]"):
        config_from_dict({"oxygen": {"boundary_mmhg": 40.0}})
    for section, key, bad in (("cells", "initial_count", 12.5), ("oxygen", "enabled", "yes"),
                              ("simulation", "device", 0)):
        with pytest.raises(ConfigError, match=f"{section}.{key}"):
            config_from_dict({section: {key: bad}})


def test_numeric_strings_are_floats_and_words_are_not():
    # reference: tests/test_config.py:44-50 (a YAML reader may hand over 7.2e6 as a string)
    cfg = config_from_dict({"oxygen": {"diffusion_um2_per_h": "7.2e6"}})
    assert cfg.oxygen.diffusion_um2_per_h == 7.2e6
    with pytest.raises(ConfigError):
        config_from_dict({"oxygen": {"diffusion_um2_per_h": "fast"}})


def test_overrides_are_typed_like_yaml_values():
    # reference: tests/test_config.py:53-63
    data = {"oxygen": {"boundary_mmHg": 38.0}}
    apply_overrides(data, ["oxygen.boundary_mmHg=150", "oxygen.grid.box_um=1200", "oxygen.enabled=false",
                           "name=culture"])
    cfg = config_from_dict(data)
    assert (cfg.oxygen.boundary_mmHg, cfg.oxygen.grid.box_um, cfg.name) == (150.0, 1200.0, "culture")
    assert cfg.oxygen.enabled is False


def test_inconsistent_setups_are_caught_and_tight_budgets_warned():
    # reference: tests/test_config.py:66-74
    with pytest.raises(ConfigError, match="does not fit"):
        config_from_dict({"cells": {"initial_count": 50_000}, "oxygen": {"grid": {"box_um": 400.0}}}).validate()
    with pytest.raises(ValueError, match="overshoot"):
        config_from_dict({"simulation": {"dt_mechanics_h": 0.1}}).validate()
    with pytest.raises(ConfigError):
        config_from_dict({"cells": {"initial_count": 10, "max_cells": 5}}).validate()
    warnings = config_from_dict({"cells": {"initial_count": 1000, "max_cells": 2000},
                                 "simulation": {"duration_h": 240.0}}).validate()
    assert any("max_cells" in w for w in warnings)


def test_disabled_oxygen_zeroes_the_lifecycle_oxygen_thresholds():
    # reference: tests/test_config.py:77-80
    params = config_from_dict({"oxygen": {"enabled": False}}).lifecycle_params()
    assert params.hypoxia_threshold == 0.0 and params.death_threshold == 0.0



def test_network_section_validation():
    # reference: tests/test_experiment.py:166-180 (input sources must be fields of the run, input
    # nodes must exist, and a network without phenotype_model = network only runs alongside the rules)
    from tests.conftest import GOLDEN

    with pytest.raises(ConfigError):
        config_from_dict({"lifecycle": {"phenotype_model": "network"}}).validate()
    data = {"network": {"enabled": True, "file": str(GOLDEN / "toy_network.bnd"),
                        "cfg": str(GOLDEN / "toy_network.cfg"),
                        "inputs": [{"node": "Signal", "source": "lactate", "threshold": 1.0}]}}
    with pytest.raises(ConfigError):
        config_from_dict(data).validate()  # no lactate field in this run
    data["network"]["inputs"][0]["source"] = "oxygen"
    data["network"]["inputs"].append({"node": "Nope", "source": "constant"})
    with pytest.raises(ConfigError):
        config_from_dict(data).validate()  # no such node
    data["network"]["inputs"].pop()
    assert any("phenotype_model = rules" in w for w in config_from_dict(data).validate())


def test_species_section_validation():
    # reference: tests/test_species.py:179-192
    with pytest.raises(ConfigError, match="unique"):
        config_from_dict({"species": [{"name": "oxygen"}]}).validate()
    with pytest.raises(ConfigError, match=r"species\[0\]"):
        config_from_dict({"species": [{"name": "glucose", "diffusion_um2_per_h": "fast"}]})
    assert any("glucose" in w for w in config_from_dict({"lifecycle": {"necrosis_requires_glucose": True}}).validate())
    # without a glucose species the lifecycle ignores the glucose rules
    params = config_from_dict({"lifecycle": {"glucose_threshold_mM": 4.0,
                                             "necrosis_requires_glucose": True}}).lifecycle_params()
    assert params.glucose_threshold == 0.0 and params.necrosis_requires_glucose is False


# The reference project's checkout, when one is on this machine (WBC_REFERENCE_ROOT names it).
REFERENCE_CONFIGS = Path(os.environ.get("WBC_REFERENCE_ROOT", "")) / "configs" if os.environ.get("WBC_REFERENCE_ROOT") \
    else None


@pytest.mark.skipif(REFERENCE_CONFIGS is None or not REFERENCE_CONFIGS.is_dir(),
                    reason="WBC_REFERENCE_ROOT does not name a checkout of the reference with its configs")
def test_reference_configuration_files_load_with_their_values():
    """Every shipped configuration of the reference loads through the YAML subset reader, with the
    values its files state (configs/*.yaml, configs/sweeps/oxygen_boundary.yaml)."""
    base = {p.name: load_config(p) for p in sorted(REFERENCE_CONFIGS.glob("*.yaml"))}
    assert set(base) == {"microc_oxygen.yaml", "tumor_in_ellipsoid.yaml", "tumor_spheroid.yaml",
                         "tumor_spheroid_metabolic.yaml", "tumor_spheroid_network.yaml"}
    for name, c in base.items():
        assert c.simulation.dt_cells_h == 0.25 and c.simulation.seed == 0 and c.cells.max_cells == 200000, name
        assert c.oxygen.grid.dx_um == 20.0, name
    assert base["tumor_spheroid.yaml"].simulation.duration_h == 168.0
    assert base["tumor_spheroid.yaml"].oxygen.boundary_mmHg == 38.0
    assert base["microc_oxygen.yaml"].oxygen.boundary_mmHg == 50.0
    ell = base["tumor_in_ellipsoid.yaml"]
    assert ell.simulation.duration_h == 96.0 and ell.geometry.shape == "ellipsoid" and ell.geometry.seed_fill
    met = base["tumor_spheroid_metabolic.yaml"]
    assert [s.boundary_value for s in met.species] == [5.0, 1.0]
    net = base["tumor_spheroid_network.yaml"]
    assert net.network.enabled and net.network.update == "asynchronous" and net.network.updates_per_step == 200
    spec = load_sweep(REFERENCE_CONFIGS / "sweeps" / "oxygen_boundary.yaml")
    assert len(list(spec.runs())) == 15  # 5 boundary values x seeds [0, 1, 2]


def test_run_directory_tables_and_metadata(tmp_path):
    """The run directory's files, CSV headers and rows, and the metadata life cycle (reference:
    io/run_output.py): the column names are the format's contract."""
    import csv
    import json

    from warpbiocell_gb300.io.run_output import METRIC_COLUMNS, PROFILE_COLUMNS, RunOutput, make_run_dir

    first = make_run_dir(tmp_path, "demo")
    second = make_run_dir(tmp_path, "demo")
    assert first != second and first.is_dir() and second.is_dir() and first.name.endswith("_demo")

    cfg = config_from_dict({"name": "demo"}).to_dict()
    out = RunOutput(first, None, cfg, "cpu", seed=5)
    assert (first / "checkpoint").is_dir() and (first / "config.yaml").exists()
    out.write_metrics({"time_h": 0.0, "cells": 10, "not_a_column": 1})
    profile = {"r_outer": np.array([20.0, 40.0]), "cells": np.array([3, 7]), "oxygen_mean": np.array([30.0, 35.0]),
               "lactate_mean": np.array([1.0, 2.0]),
               **{f"fraction_{s}": np.array([0.5, 0.25]) for s in ("proliferative", "quiescent", "hypoxic", "dead")}}
    out.write_profile(1.5, profile)
    meta = json.loads((first / "metadata.json").read_text())
    assert meta["status"] == "running" and meta["seed"] == 5 and meta["config"]["name"] == "demo"
    out.finish("completed", 2.0, {"cells": 10})
    meta = json.loads((first / "metadata.json").read_text())
    assert meta["status"] == "completed" and meta["wall_s"] == 2.0 and meta["summary"] == {"cells": 10}
    assert out.checkpoint_path(1.5).name == "state_0001.50h.npz"

    with (first / "metrics.csv").open() as f:
        rows = list(csv.DictReader(f))
    assert list(rows[0]) == METRIC_COLUMNS and rows[0]["cells"] == "10" and rows[0]["wall_s"] == ""
    with (first / "profiles.csv").open() as f:
        rows = list(csv.DictReader(f))
    assert list(rows[0]) == PROFILE_COLUMNS and len(rows) == 2
    assert rows[1]["shell"] == "1" and rows[1]["cells"] == "7" and rows[1]["r_outer_um"] == "40.0"
    assert rows[0]["glucose_mean_mM"] == "" and rows[0]["lactate_mean_mM"] == "1.0"
    assert rows[0]["time_h"] == "1.5" and rows[0]["fraction_dead"] == "0.5"

"""Run directory layout (reference: io/run_output.py, whose file names, column names and metadata
keys these keep)::

    <run>/config.yaml     the input configuration (verbatim copy, or the resolved values)
    <run>/metadata.json   resolved config, seed, versions, device, timing, status, summary
    <run>/metrics.csv     one row per metrics interval (METRIC_COLUMNS)
    <run>/profiles.csv    radial profiles, one row per shell per profile interval (PROFILE_COLUMNS)
    <run>/checkpoint/     state_<time>h.npz

Each CSV table is flushed after every row, so an interrupted run still leaves usable data.
"""

from __future__ import annotations

import csv
import datetime as dt
import itertools
import json
import platform
import shutil
import subprocess
from pathlib import Path

import torch

import warpbiocell_gb300
from warpbiocell_gb300.simulation import yaml_subset

METRIC_COLUMNS = [
    "time_h", "cells", "living_cells", "dead_cells", "proliferative_cells", "quiescent_cells", "hypoxic_cells",
    "mean_radius_um", "spheroid_radius_um", "necrotic_radius_um", "hypoxic_radius_um",
    "non_proliferative_radius_um", "viable_rim_um", "proliferating_rim_um", "oxygen_cells_mean_mmHg",
    "oxygen_cells_min_mmHg", "oxygen_grid_mean_mmHg", "oxygen_grid_min_mmHg", "glucose_cells_mean_mM",
    "glucose_cells_min_mM", "lactate_cells_mean_mM", "lactate_cells_max_mM", "network_proliferation_cells",
    "network_apoptosis_cells", "network_growth_arrest_cells", "network_necrosis_cells", "field_sweeps",
    "cells_outside_grid", "cells_outside_tissue", "wall_s",
]

# profiles.csv column -> key of the radial profile it is read from; None for the columns the
# writer fills itself; the optional species are left empty when the profile has no such key
_PROFILE_SOURCE = {
    "time_h": None,
    "shell": None,
    "r_outer_um": "r_outer",
    "cells": "cells",
    "oxygen_mean_mmHg": "oxygen_mean",
    "glucose_mean_mM": "glucose_mean",
    "lactate_mean_mM": "lactate_mean",
    "fraction_proliferative": "fraction_proliferative",
    "fraction_quiescent": "fraction_quiescent",
    "fraction_hypoxic": "fraction_hypoxic",
    "fraction_dead": "fraction_dead",
}
_OPTIONAL_PROFILE_KEYS = {"glucose_mean", "lactate_mean"}
PROFILE_COLUMNS = list(_PROFILE_SOURCE)


def git_commit() -> str | None:
    """HEAD of the checkout the package was imported from, or None outside a git checkout."""
    checkout = Path(warpbiocell_gb300.__file__).resolve().parent.parent
    try:
        head = subprocess.check_output(["git", "rev-parse", "HEAD"], cwd=checkout, stderr=subprocess.DEVNULL,
                                       text=True, timeout=5)
    except (OSError, subprocess.SubprocessError):
        return None
    return head.strip() or None


def make_run_dir(base: str | Path, name: str) -> Path:
    """Create and return ``<base>/<local time>_<name>``, numbered ``_1``, ``_2`` ... when taken."""
    stem = f"{dt.datetime.now():%Y-%m-%dT%H-%M-%S}_{name}"
    Path(base).mkdir(parents=True, exist_ok=True)
    for k in itertools.count():
        path = Path(base) / (stem if k == 0 else f"{stem}_{k}")
        try:
            path.mkdir()
        except FileExistsError:
            continue
        return path


def _now() -> str:
    return dt.datetime.now(dt.timezone.utc).isoformat()


def _describe_device(device) -> dict:
    device = torch.device(device)
    record = {"alias": str(device), "is_cuda": device.type == "cuda"}
    if record["is_cuda"] and torch.cuda.is_available():
        record["name"] = torch.cuda.get_device_name(device)
    return record


class _CsvTable:
    """A CSV file with a fixed header, flushed after every row."""

    def __init__(self, path: Path, columns: list[str]):
        self._file = path.open("w", newline="")
        self._writer = csv.DictWriter(self._file, fieldnames=columns)
        self._writer.writeheader()
        self._file.flush()

    def append(self, rows) -> None:
        self._writer.writerows(rows)
        self._file.flush()

    def close(self) -> None:
        self._file.close()


class RunOutput:
    """Writes one run's directory: configuration, metadata, metrics and profile tables, and the
    checkpoint paths."""

    def __init__(self, directory: Path, config_path: Path | None, config_dict: dict, device, seed: int):
        self.directory = Path(directory)
        (self.directory / "checkpoint").mkdir(parents=True, exist_ok=True)
        if config_path is None:
            self._dump_config(config_dict)
        else:
            shutil.copyfile(config_path, self.directory / "config.yaml")
        self.metadata = dict(
            name=config_dict.get("name"), status="running", started=_now(), finished=None, wall_s=None, seed=seed,
            warpbiocell_gb300_version=warpbiocell_gb300.__version__, git_commit=git_commit(),
            torch_version=torch.__version__, device=_describe_device(device), platform=platform.platform(),
            python=platform.python_version(), config=config_dict, warnings=[], summary=None,
        )
        self._metrics = _CsvTable(self.directory / "metrics.csv", METRIC_COLUMNS)
        self._profiles = _CsvTable(self.directory / "profiles.csv", PROFILE_COLUMNS)
        self.write_metadata()

    def _dump_config(self, config_dict: dict) -> None:
        (self.directory / "config.yaml").write_text(yaml_subset.safe_dump(config_dict))

    def write_metrics(self, row: dict) -> None:
        """One metrics row; columns the row lacks are left empty."""
        self._metrics.append([{column: row.get(column, "") for column in METRIC_COLUMNS}])

    def write_profile(self, time_h: float, profile: dict) -> None:
        """One row per shell of a radial profile (``metrics.population.radial_profile``)."""
        rows = []
        for shell in range(len(profile["r_outer"])):
            row = {"time_h": time_h, "shell": shell}
            for column, key in _PROFILE_SOURCE.items():
                if key is None:
                    continue
                if key not in profile and key in _OPTIONAL_PROFILE_KEYS:
                    row[column] = ""
                else:
                    value = profile[key][shell]
                    row[column] = int(value) if key == "cells" else float(value)
            rows.append(row)
        self._profiles.append(rows)

    def checkpoint_path(self, time_h: float) -> Path:
        return self.directory / "checkpoint" / f"state_{time_h:07.2f}h.npz"

    def write_metadata(self) -> None:
        (self.directory / "metadata.json").write_text(json.dumps(self.metadata, indent=2, default=str))

    def write_config(self, config_dict: dict) -> None:
        """Replace the recorded configuration (drivers that assemble it piece by piece)."""
        self.metadata["config"] = config_dict
        self.metadata["name"] = config_dict.get("name", self.metadata.get("name"))
        self._dump_config(config_dict)
        self.write_metadata()

    def finish(self, status: str, wall_s: float, summary: dict | None) -> None:
        """Record the outcome and close the tables."""
        self.metadata.update(status=status, finished=_now(), wall_s=wall_s, summary=summary)
        self.write_metadata()
        self._metrics.close()
        self._profiles.close()

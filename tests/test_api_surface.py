"""The drop-in surface (host logic, no device): every public function, class, method and dataclass
field of the reference's model API (recorded from its source in tests/golden/api_surface.json by
tests/golden/make_api_surface.py) exists in warpbiocell_gb300 under the same module path, with the
same parameter names in the same order. Extra trailing parameters are allowed (they all have
defaults, so the reference's calls still bind)."""

import dataclasses
import importlib
import inspect
import json

import pytest

from conftest import GOLDEN

SURFACE = json.loads((GOLDEN / "api_surface.json").read_text())


def _names(fn) -> list[str]:
    out = []
    for p in inspect.signature(fn).parameters.values():
        if p.kind == p.VAR_POSITIONAL:
            out.append("*" + p.name)
        elif p.kind == p.VAR_KEYWORD:
            out.append("**" + p.name)
        else:
            out.append(p.name)
    return out


def _extra_have_defaults(fn, n_ref: int) -> bool:
    params = list(inspect.signature(fn).parameters.values())[n_ref:]
    return all(p.default is not p.empty or p.kind in (p.VAR_POSITIONAL, p.VAR_KEYWORD) for p in params)


def test_surface_fixture_covers_the_model_api():
    assert len(SURFACE) == 28
    assert sum(len(v) for v in SURFACE.values()) >= 100
    for key in ("cells.state", "cells.mechanics", "cells.lifecycle", "spatial.neighbors", "fields.oxygen",
                "fields.diffusion", "network.runtime", "simulation.simulator", "simulation.experiment"):
        assert SURFACE[key], key


@pytest.mark.parametrize("module", sorted(SURFACE))
def test_module_matches_reference_surface(module):
    m = importlib.import_module("warpbiocell_gb300." + module)
    problems = []
    for name, info in SURFACE[module].items():
        if not hasattr(m, name):
            problems.append(f"missing {name}")
            continue
        obj = getattr(m, name)
        if info["kind"] == "function":
            ours = _names(obj)
            if ours[:len(info["params"])] != info["params"] or not _extra_have_defaults(obj, len(info["params"])):
                problems.append(f"{name}: reference {info['params']}, here {ours}")
            continue
        for meth, mi in info["methods"].items():
            if not hasattr(obj, meth):
                problems.append(f"missing {name}.{meth}")
                continue
            attr = inspect.getattr_static(obj, meth)
            if mi["property"]:
                if not isinstance(attr, property) and not dataclasses.is_dataclass(obj):
                    problems.append(f"{name}.{meth} is not a property")
                continue
            fn = attr.__func__ if isinstance(attr, (staticmethod, classmethod)) else attr
            ours = _names(fn)
            if ours[:len(mi["params"])] != mi["params"] or not _extra_have_defaults(fn, len(mi["params"])):
                problems.append(f"{name}.{meth}: reference {mi['params']}, here {ours}")
        if info["fields"] and dataclasses.is_dataclass(obj):
            ours = [f.name for f in dataclasses.fields(obj)]
            missing = [f for f in info["fields"] if f not in ours]
            if missing:
                problems.append(f"{name}: missing fields {missing}")
    assert not problems, "\n".join(problems)

"""Record the reference's public Python model API as a fixture: module by module, every public
function with its parameter names, every public class with its methods (parameter names, and
whether a method is a property) and its annotated (dataclass) fields.

The reference's modules import NVIDIA Warp, which is absent here, so they are read as source
(Python's ``ast``), not imported. The modules are the ones a caller of the coupled cell step uses:
cells, spatial, fields, network, simulation, geometry, io and metrics (the command-line runners,
export, visualisation and the Warp kernels themselves are not part of the drop-in surface).

Run from the repository root:  python tests/golden/make_api_surface.py [/path/to/reference]
Output (committed): tests/golden/api_surface.json. The tests never read the reference.
"""

from __future__ import annotations

import ast
import json
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
# The reference project's checkout: the first argument, else $WBC_REFERENCE_ROOT.
_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("WBC_REFERENCE_ROOT")
if not _root:
    sys.exit(f"usage: {Path(__file__).name} <reference checkout> (or set WBC_REFERENCE_ROOT)")
REFERENCE = Path(_root)
MODULES = ["device.py", "cells/state.py", "cells/mechanics.py", "cells/lifecycle.py", "cells/model.py",
           "cells/initialization.py",
           "spatial/neighbors.py", "fields/densities.py", "fields/diffusion.py", "fields/metabolism.py",
           "fields/oxygen.py", "fields/scalar_field.py", "fields/species.py", "network/expression.py",
           "network/model.py", "network/runtime.py", "simulation/config.py", "simulation/experiment.py",
           "simulation/simulator.py", "simulation/sweep.py", "geometry/region.py", "geometry/seeding.py",
           "geometry/shapes.py", "geometry/masks.py", "io/checkpoints.py", "io/run_output.py", "metrics/population.py",
           "metrics/timeseries.py"]


def _params(fn: ast.FunctionDef) -> list[str]:
    a = fn.args
    names = [x.arg for x in a.posonlyargs + a.args]
    if a.vararg:
        names.append("*" + a.vararg.arg)
    names += [x.arg for x in a.kwonlyargs]
    if a.kwarg:
        names.append("**" + a.kwarg.arg)
    return names


def _decorators(fn: ast.FunctionDef) -> list[str]:
    out = []
    for d in fn.decorator_list:
        out.append(d.id if isinstance(d, ast.Name) else d.attr if isinstance(d, ast.Attribute) else "")
    return out


def surface(root: Path) -> dict:
    out = {}
    for rel in MODULES:
        tree = ast.parse((root / "src" / "warpbiocell" / rel).read_text())
        mod = {}
        for node in tree.body:
            if isinstance(node, (ast.FunctionDef, ast.AsyncFunctionDef)) and not node.name.startswith("_"):
                mod[node.name] = {"kind": "function", "params": _params(node)}
            elif isinstance(node, ast.ClassDef) and not node.name.startswith("_"):
                methods, fields = {}, []
                for b in node.body:
                    if isinstance(b, (ast.FunctionDef, ast.AsyncFunctionDef)) and (
                            not b.name.startswith("_") or b.name == "__init__"):
                        deco = _decorators(b)
                        methods[b.name] = {"params": _params(b), "property": "property" in deco,
                                           "classmethod": "classmethod" in deco,
                                           "staticmethod": "staticmethod" in deco}
                    elif isinstance(b, ast.AnnAssign) and isinstance(b.target, ast.Name):
                        fields.append(b.target.id)
                mod[node.name] = {"kind": "class", "methods": methods, "fields": fields}
        out[rel[:-3].replace("/", ".")] = mod
    return out


if __name__ == "__main__":
    data = surface(REFERENCE)
    (HERE / "api_surface.json").write_text(json.dumps(data, indent=1, sort_keys=True) + "\n")
    print(f"{sum(len(v) for v in data.values())} public names in {len(data)} modules")

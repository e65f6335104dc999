"""Tissue regions: signed-distance fields on a grid, synthetic shapes and seeding
(reference: geometry/)."""

from warpbiocell_gb300.geometry.region import TissueRegion, node_gradient
from warpbiocell_gb300.geometry.seeding import CellBudgetError, fill_region
from warpbiocell_gb300.geometry.shapes import Ellipsoid, Sphere, Union, evaluate_on_grid

__all__ = ["TissueRegion", "node_gradient", "CellBudgetError", "fill_region", "Ellipsoid", "Sphere", "Union",
           "evaluate_on_grid"]

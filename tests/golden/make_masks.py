"""Generate tests/golden/masks.npz from the reference's own mask helpers.

The reference's ``geometry/masks.py`` (``sdf_from_mask``, ``resample_nearest``) is numpy + scipy;
it reaches Warp only through imports, which the stand-in of ``make_golden.py`` satisfies.
Each case records a voxel mask, its spacing, the signed distance the reference computes on the
mask's own grid, and that distance resampled (nearest voxel) onto a simulation grid with the
reference's far-field fill value.

Run from the repository root:  python tests/golden/make_masks.py [/path/to/reference]
Output (committed): tests/golden/masks.npz. The tests never import the reference.
"""

from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# The reference project's checkout: the first argument, else $WBC_REFERENCE_ROOT.
_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("WBC_REFERENCE_ROOT")
if not _root:
    sys.exit(f"usage: {Path(__file__).name} <reference checkout> (or set WBC_REFERENCE_ROOT)")
REFERENCE = Path(_root)


def _cases():
    """(name, mask, voxel size, mask origin, grid origin, grid dx, grid shape)."""
    n, voxel = 24, 10.0
    c = (np.arange(n) - (n - 1) / 2.0) * voxel
    x, y, z = np.meshgrid(c, c, c, indexing="ij")
    yield "sphere", np.sqrt(x**2 + y**2 + z**2) < 90.0, voxel, (c[0],) * 3, (-140.0,) * 3, 20.0, (15, 15, 15)
    # anisotropic voxels, an off-centre ellipsoid, a grid that only partly overlaps the mask
    sx, sy, sz = 8.0, 12.0, 15.0
    nx, ny, nz = 30, 22, 18
    x, y, z = np.meshgrid(np.arange(nx) * sx, np.arange(ny) * sy, np.arange(nz) * sz, indexing="ij")
    ell = ((x - 120.0) / 90.0) ** 2 + ((y - 130.0) / 70.0) ** 2 + ((z - 120.0) / 80.0) ** 2 < 1.0
    yield "ellipsoid_anisotropic", ell, (sx, sy, sz), (-100.0, -120.0, -110.0), (-150.0, -150.0, -150.0), 25.0, \
        (13, 12, 11)
    # two touching blobs and a one-voxel speck (disconnected components)
    m = np.zeros((20, 20, 20), dtype=bool)
    m[3:9, 4:12, 5:11] = True
    m[8:16, 9:17, 8:15] = True
    m[17, 2, 17] = True
    yield "two_blobs_and_speck", m, 5.0, (0.0, 0.0, 0.0), (-10.0, -10.0, -10.0), 7.5, (16, 16, 16)


def main() -> None:
    sys.path.insert(0, str(HERE))
    from make_golden import _install_warp_stand_in

    _install_warp_stand_in()
    sys.path.insert(0, str(REFERENCE / "src"))
    from warpbiocell.fields.scalar_field import GridGeometry
    from warpbiocell.geometry.masks import resample_nearest, sdf_from_mask

    out = {}
    names = []
    for name, mask, voxel, mask_origin, origin, dx, shape in _cases():
        sdf = sdf_from_mask(mask, voxel)
        far = float(np.abs(sdf).max()) + 10.0 * float(np.max(np.atleast_1d(voxel)))
        geom = GridGeometry(origin=origin, dx=dx, shape=shape)
        names.append(name)
        out[f"{name}_mask"] = mask
        out[f"{name}_voxel"] = np.array(np.broadcast_to(np.asarray(voxel, dtype=float), (3,)))
        out[f"{name}_mask_origin"] = np.array(mask_origin, dtype=float)
        out[f"{name}_grid"] = np.array([*origin, dx, *shape], dtype=float)
        out[f"{name}_sdf"] = sdf
        out[f"{name}_far"] = np.array(far)
        out[f"{name}_resampled"] = resample_nearest(sdf, voxel, mask_origin, geom, fill=far)
    out["cases"] = np.array(names)
    np.savez_compressed(HERE / "masks.npz", **out)
    print("wrote", HERE / "masks.npz", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()

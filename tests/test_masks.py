"""Tissue regions from voxel masks on the host (reference: tests/test_masks.py,
geometry/masks.py): the signed distance and its resampling are bit-identical to the reference's
own helpers on the fixtures of tests/golden/make_masks.py; the reference's analytical cases hold;
NIfTI-1 label images written byte by byte from the format's header layout read back exactly."""

import gzip
import struct

import numpy as np
import pytest

from warpbiocell_gb300.fields.scalar_field import GridGeometry
from warpbiocell_gb300.geometry.masks import (load_nifti_mask, read_nifti, region_from_mask, resample_nearest,
                                              sdf_from_mask)
from warpbiocell_gb300.geometry.shapes import Sphere

pytest.importorskip("scipy")


def test_signed_distance_and_resampling_equal_the_reference_bitwise(golden):
    g = golden("masks")
    for name in g["cases"]:
        name = str(name)
        mask, voxel, mask_origin = g[f"{name}_mask"], g[f"{name}_voxel"], tuple(g[f"{name}_mask_origin"])
        voxel = float(voxel[0]) if np.all(voxel == voxel[0]) else tuple(voxel)
        sdf = sdf_from_mask(mask, voxel)
        assert sdf.dtype == np.float32
        np.testing.assert_array_equal(sdf, g[f"{name}_sdf"], err_msg=name)
        grid = g[f"{name}_grid"]
        geom = GridGeometry(origin=tuple(grid[:3]), dx=float(grid[3]), shape=tuple(int(v) for v in grid[4:]))
        far = float(g[f"{name}_far"])
        np.testing.assert_array_equal(resample_nearest(sdf, voxel, mask_origin, geom, fill=far),
                                      g[f"{name}_resampled"], err_msg=name)
        region = region_from_mask(mask, voxel, geom, mask_origin=mask_origin, device=None, name=name)
        np.testing.assert_array_equal(region.sdf_numpy(), g[f"{name}_resampled"], err_msg=name)


def _voxel_sphere(n=40, voxel=10.0, radius=150.0):
    c = (np.arange(n) - (n - 1) / 2.0) * voxel
    x, y, z = np.meshgrid(c, c, c, indexing="ij")
    return np.sqrt(x**2 + y**2 + z**2) < radius, c[0], np.sqrt(x**2 + y**2 + z**2) - radius


def test_sdf_of_a_voxel_sphere_is_within_a_voxel_of_the_exact_distance():
    # reference: tests/test_masks.py:19-29
    mask, _, exact = _voxel_sphere()
    sdf = sdf_from_mask(mask, 10.0)
    assert np.array_equal(sdf < 0, mask)
    assert np.abs(sdf - exact).max() < 15.0
    assert np.abs(sdf - exact)[np.abs(exact) < 50.0].mean() < 5.0
    with pytest.raises(ValueError):
        sdf_from_mask(np.zeros((4, 4, 4), dtype=bool), 10.0)
    with pytest.raises(ValueError):
        sdf_from_mask(np.ones((4, 4), dtype=bool), 10.0)
    with pytest.raises(ValueError):
        sdf_from_mask(np.ones((4, 4, 4), dtype=bool), (10.0, -1.0, 10.0))


def test_region_from_mask_on_the_simulation_grid():
    # reference: tests/test_masks.py:32-40
    mask, origin, _ = _voxel_sphere()
    geom = GridGeometry.centered_cube(400.0, 20.0)
    region = region_from_mask(mask, 10.0, geom, mask_origin=(origin,) * 3)
    assert abs(region.volume() / Sphere(radius=150.0).volume - 1.0) < 0.1
    pts = np.array([[0.0, 0.0, 0.0], [140.0, 0.0, 0.0], [160.0, 0.0, 0.0], [0.0, 195.0, 0.0]])
    np.testing.assert_array_equal(region.contains(pts), [True, True, False, False])
    # nodes beyond the mask's extent are far outside
    far_geom = GridGeometry.centered_cube(1000.0, 50.0)
    sdf = region_from_mask(mask, 10.0, far_geom, mask_origin=(origin,) * 3).sdf_numpy()
    assert sdf[0, 0, 0] > np.abs(sdf_from_mask(mask, 10.0)).max()


# ---- NIfTI-1, written from the header layout (348 bytes; dim at 40, datatype 70, bitpix 72,
# pixdim 76, vox_offset 108, scl_slope/scl_inter 112, magic 344) -------------------------------------
_CODES = {np.dtype("u1"): 2, np.dtype("i2"): 4, np.dtype("i4"): 8, np.dtype("f4"): 16, np.dtype("f8"): 64}


def _header(data, pixdim_mm, order, magic, vox_offset, slope=0.0, inter=0.0):
    hdr = bytearray(348)
    struct.pack_into(order + "i", hdr, 0, 348)
    dims = [data.ndim, *data.shape] + [1] * (7 - data.ndim)
    struct.pack_into(order + "8h", hdr, 40, *dims)
    struct.pack_into(order + "h", hdr, 70, _CODES[data.dtype.newbyteorder("=")])
    struct.pack_into(order + "h", hdr, 72, 8 * data.dtype.itemsize)
    pix = [1.0, *pixdim_mm] + [0.0] * (7 - len(pixdim_mm))
    struct.pack_into(order + "8f", hdr, 76, *pix)
    struct.pack_into(order + "f", hdr, 108, float(vox_offset))
    struct.pack_into(order + "2f", hdr, 112, slope, inter)
    hdr[344:348] = magic
    return bytes(hdr)


def _write_single(path, data, pixdim_mm, order="<", compress=False, **kw):
    body = data.astype(data.dtype.newbyteorder(order)).tobytes(order="F")
    raw = _header(data, pixdim_mm, order, b"n+1\x00", 352, **kw) + b"\x00" * 4 + body
    path.write_bytes(gzip.compress(raw) if compress else raw)


def test_nifti_label_image_round_trip(tmp_path):
    # reference: tests/test_masks.py:43-56 (20 um voxels stored as 0.02 mm, label 2)
    mask, origin, _ = _voxel_sphere(n=30, voxel=20.0, radius=120.0)
    labels = np.where(mask, 2, 0).astype(np.int16)
    labels[0, 0, 0] = 5  # another label
    path = tmp_path / "tumour.nii.gz"
    _write_single(path, labels, (0.02, 0.02, 0.02), compress=True)
    loaded, voxel = load_nifti_mask(path, label=2)
    np.testing.assert_array_equal(loaded, mask)
    np.testing.assert_allclose(voxel, (20.0, 20.0, 20.0), rtol=1e-5)
    any_label, _ = load_nifti_mask(path)
    assert any_label.sum() == mask.sum() + 1
    region = region_from_mask(loaded, voxel, GridGeometry.centered_cube(400.0, 20.0), mask_origin=(origin,) * 3)
    assert abs(region.volume() / Sphere(radius=120.0).volume - 1.0) < 0.15


@pytest.mark.parametrize("order", ["<", ">"])
@pytest.mark.parametrize("dtype", ["u1", "i2", "i4", "f4", "f8"])
def test_nifti_voxel_order_byte_order_and_types(tmp_path, order, dtype):
    rng = np.random.default_rng(3)
    data = rng.integers(0, 7, size=(5, 4, 3)).astype(dtype)
    path = tmp_path / "x.nii"
    _write_single(path, data, (0.5, 0.25, 2.0), order=order)
    values, pixdim = read_nifti(path)
    np.testing.assert_array_equal(values, data)  # [i, j, k] with i fastest on disk
    assert pixdim == (0.5, 0.25, 2.0)


def test_nifti_scaling_and_header_image_pairs(tmp_path):
    data = np.arange(24, dtype=np.int16).reshape(2, 3, 4)
    path = tmp_path / "s.nii"
    _write_single(path, data, (1.0, 1.0, 1.0), slope=2.0, inter=-1.0)
    np.testing.assert_array_equal(read_nifti(path)[0], 2.0 * data - 1.0)
    # header and voxels in two files
    (tmp_path / "p.hdr").write_bytes(_header(data, (0.01, 0.01, 0.01), "<", b"ni1\x00", 0))
    (tmp_path / "p.img").write_bytes(data.tobytes(order="F"))
    mask, voxel = load_nifti_mask(tmp_path / "p.hdr", label=7)
    assert mask.sum() == 1 and mask[0, 1, 3]  # data[i, j, k] = 12 i + 4 j + k
    np.testing.assert_allclose(voxel, (10.0, 10.0, 10.0), rtol=1e-5)


def test_nifti_rejects_what_it_cannot_read(tmp_path):
    data = np.zeros((2, 2, 2), dtype=np.int16)
    bad = tmp_path / "bad.nii"
    raw = bytearray(_header(data, (1.0, 1.0, 1.0), "<", b"n+1\x00", 352) + b"\x00" * 4 + data.tobytes())
    raw[344:348] = b"xxxx"
    bad.write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="magic"):
        read_nifti(bad)
    two = tmp_path / "two.nii"
    two.write_bytes(struct.pack("<i", 540) + b"\x00" * 600)
    with pytest.raises(ValueError, match="NIfTI-2"):
        read_nifti(two)
    short = tmp_path / "short.nii"
    short.write_bytes(_header(data, (1.0, 1.0, 1.0), "<", b"n+1\x00", 352))  # no voxels
    with pytest.raises(ValueError, match="do not fit"):
        read_nifti(short)


def test_experiment_builds_a_region_from_a_mask_file(tmp_path):
    # reference: simulation/experiment.py:141-145, with the mask file named relative to the config
    from warpbiocell_gb300.simulation.config import config_from_dict
    from warpbiocell_gb300.simulation.experiment import Experiment

    mask, origin, _ = _voxel_sphere(n=30, voxel=20.0, radius=120.0)
    _write_single(tmp_path / "lesion.nii.gz", np.where(mask, 3, 0).astype(np.int16), (0.02, 0.02, 0.02),
                  compress=True)
    cfg = config_from_dict({"geometry": {"enabled": True, "shape": "mask", "mask_file": "lesion.nii.gz",
                                         "mask_label": 3, "mask_origin_um": [origin] * 3},
                            "cells": {"max_cells": 20000}, "oxygen": {"grid": {"box_um": 400.0}}})
    exp = Experiment.__new__(Experiment)  # the region needs no device until it is used
    exp.config, exp.base_dir, exp.device = cfg, tmp_path, None
    region = exp._build_region()
    assert region.name == "lesion.nii.gz"
    assert abs(region.volume() / Sphere(radius=120.0).volume - 1.0) < 0.15

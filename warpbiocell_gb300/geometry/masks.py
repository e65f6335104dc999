"""Tissue regions from voxel masks (reference: geometry/masks.py).

``sdf_from_mask`` turns a binary voxel mask into a signed distance (negative inside) with two
Euclidean distance transforms, ``region_from_mask`` resamples it onto a simulation grid as a
:class:`TissueRegion`, and ``load_nifti_mask`` reads a NIfTI-1 label image. All of this is host
work done once per run; the region then lives on the device like any other.

The NIfTI-1 reader is this package's own (nibabel is not a dependency): single-file ``.nii`` and
``.hdr``/``.img`` pairs, optionally gzip-compressed, either byte order, the integer and float
voxel types, and the header's scaling (``scl_slope``/``scl_inter``). Voxel sizes are taken in
millimetres, as the reference does, and returned in micrometres.
"""

from __future__ import annotations

import gzip
import struct
from pathlib import Path

import numpy as np

from warpbiocell_gb300.fields.scalar_field import GridGeometry
from warpbiocell_gb300.geometry.region import TissueRegion


def _spacing(voxel_size) -> np.ndarray:
    s = np.asarray(voxel_size, dtype=np.float64)
    s = np.broadcast_to(s, (3,)) if s.ndim == 0 else s
    if s.shape != (3,) or np.any(s <= 0.0):
        raise ValueError(f"voxel size must be one positive value or three, got {voxel_size!r}")
    return s


def sdf_from_mask(mask: np.ndarray, voxel_size) -> np.ndarray:
    """Signed distance [um] on the mask's own voxel grid, negative inside, float32.

    Inside voxels get minus their distance to the nearest outside voxel, outside voxels their
    distance to the nearest inside voxel; both less half the smallest spacing, which puts the
    zero level on the faces between inside and outside voxels (reference: geometry/masks.py:21-37).
    """
    from scipy.ndimage import distance_transform_edt

    mask = np.asarray(mask).astype(bool)
    if mask.ndim != 3:
        raise ValueError(f"mask must be a 3-D array, got {mask.ndim} dimensions")
    if not mask.any():
        raise ValueError("mask is empty")
    spacing = tuple(float(s) for s in _spacing(voxel_size))
    to_tissue = distance_transform_edt(~mask, sampling=spacing)
    to_exterior = distance_transform_edt(mask, sampling=spacing)
    half = 0.5 * min(spacing)
    return np.where(mask, -(to_exterior - half), to_tissue - half).astype(np.float32)


def resample_nearest(values: np.ndarray, voxel_size, mask_origin, geometry: GridGeometry, fill: float) -> np.ndarray:
    """``values`` (on the mask grid, voxel (0,0,0) at ``mask_origin`` [um]) at the nearest mask voxel
    of every node of ``geometry``; ``fill`` where a node falls outside the mask's extent
    (reference: geometry/masks.py:40-51). The nearest index is rounded half to even, per axis."""
    spacing = _spacing(voxel_size)
    origin = np.asarray(mask_origin, dtype=np.float64)
    index, valid = [], []
    for a, coords in enumerate(geometry.node_coordinates()):
        i = np.rint((coords - origin[a]) / spacing[a]).astype(np.int64)
        ok = (i >= 0) & (i < values.shape[a])
        index.append(np.where(ok, i, 0))
        valid.append(ok)
    gathered = np.asarray(values)[np.ix_(*index)].astype(np.float32)
    inside = valid[0][:, None, None] & valid[1][None, :, None] & valid[2][None, None, :]
    return np.where(inside, gathered, np.float32(fill)).astype(np.float32)


def region_from_mask(mask: np.ndarray, voxel_size, geometry: GridGeometry,
                     mask_origin: tuple[float, float, float] = (0.0, 0.0, 0.0), device=None,
                     name: str = "mask") -> TissueRegion:
    """A :class:`TissueRegion` on ``geometry`` from a binary mask whose voxel (0,0,0) sits at
    ``mask_origin`` [um]; nodes beyond the mask get a distance farther than any inside it
    (reference: geometry/masks.py:54-65)."""
    sdf = sdf_from_mask(mask, voxel_size)
    far = float(np.abs(sdf).max()) + 10.0 * float(np.max(np.atleast_1d(voxel_size)))
    return TissueRegion(geometry, resample_nearest(sdf, voxel_size, mask_origin, geometry, fill=far), device=device,
                        name=name)


# ---- NIfTI-1 -------------------------------------------------------------------------------------
# Header fields used here (byte offset, struct format): the NIfTI-1 header is 348 bytes.
_NIFTI_TYPES = {2: "u1", 4: "i2", 8: "i4", 16: "f4", 64: "f8", 256: "i1", 512: "u2", 768: "u4", 1024: "i8",
                1280: "u8"}


def _read_bytes(path: Path) -> bytes:
    raw = path.read_bytes()
    return gzip.decompress(raw) if raw[:2] == b"\x1f\x8b" else raw


def read_nifti(path: str | Path) -> tuple[np.ndarray, tuple[float, ...]]:
    """Voxel array (indexed [i, j, k, ...], scaled as the header says) and ``pixdim[1:]`` of a
    NIfTI-1 image."""
    path = Path(path)
    header = _read_bytes(path)
    if len(header) < 348:
        raise ValueError(f"{path}: too short for a NIfTI-1 header")
    for order in ("<", ">"):
        size = struct.unpack_from(order + "i", header, 0)[0]
        if size in (348, 540):
            break
    else:
        raise ValueError(f"{path}: not a NIfTI file (header size field {size})")
    if size == 540:
        raise ValueError(f"{path}: NIfTI-2 images are not supported")
    magic = header[344:348]
    if magic not in (b"n+1\x00", b"ni1\x00"):
        raise ValueError(f"{path}: bad NIfTI-1 magic {magic!r}")
    dim = struct.unpack_from(order + "8h", header, 40)
    ndim = dim[0]
    if not 1 <= ndim <= 7:
        raise ValueError(f"{path}: bad dimension count {ndim}")
    shape = tuple(int(d) for d in dim[1:1 + ndim])
    datatype = struct.unpack_from(order + "h", header, 70)[0]
    if datatype not in _NIFTI_TYPES:
        raise ValueError(f"{path}: unsupported NIfTI datatype {datatype}")
    pixdim = struct.unpack_from(order + "8f", header, 76)
    vox_offset = int(struct.unpack_from(order + "f", header, 108)[0])
    slope, inter = struct.unpack_from(order + "2f", header, 112)
    if magic == b"n+1\x00":
        data, start = header, vox_offset
    else:  # header and voxels in two files: x.hdr[.gz] + x.img[.gz]
        img = path.with_name(path.name.replace(".hdr", ".img"))
        data, start = _read_bytes(img), vox_offset
    dtype = np.dtype(order + _NIFTI_TYPES[datatype])
    count = int(np.prod(shape))
    if start + count * dtype.itemsize > len(data):
        raise ValueError(f"{path}: {count} voxels of {dtype} do not fit in the file")
    values = np.frombuffer(data, dtype=dtype, count=count, offset=start).reshape(shape, order="F")
    if np.isfinite(slope) and slope != 0.0 and (slope, inter) != (1.0, 0.0):
        values = values * np.float64(slope) + np.float64(inter)
    return np.array(values), tuple(float(p) for p in pixdim[1:1 + ndim])


def load_nifti_mask(path: str | Path, label: int | None = None) -> tuple[np.ndarray, tuple[float, float, float]]:
    """Binary mask (voxels equal to ``label``, or all non-zero voxels) and voxel size [um] of a
    NIfTI-1 label image whose voxel sizes are in millimetres (reference: geometry/masks.py:68-80)."""
    data, pixdim = read_nifti(path)
    mask = (data == label) if label is not None else (data > 0)
    if len(pixdim) < 3:
        raise ValueError(f"{path}: a mask needs three spatial dimensions, got {len(pixdim)}")
    return mask, tuple(1000.0 * v for v in pixdim[:3])

"""ctypes binding of libwbc_gb300.so (the C-ABI declared in include/wbc.h).

There is no CPU fallback: every compute entry point needs the library and a CUDA device, and
both are checked loudly. Arrays are torch tensors on a CUDA device; only their data pointers
and the current torch stream cross the boundary.
"""

from __future__ import annotations

import ctypes
import threading
from ctypes import POINTER, c_float, c_int32, c_int64, c_size_t, c_void_p
from pathlib import Path

import torch

from warpbiocell_gb300._build import library_path

WBC_OK = 0
WBC_ERR_INVALID = -1
WBC_ERR_CAPACITY = -2
WBC_ERR_CUDA = -4
WBC_ERR_TIMEOUT = -5
WBC_ERR_WORKSPACE = -6


class LibraryError(RuntimeError):
    """The native library is missing, failed to load, or a call returned an error status."""


class NeighborGridC(ctypes.Structure):
    _fields_ = [
        ("dim", c_int32),
        ("cell_size", c_float),
        ("bucket_count", c_void_p),
        ("bucket_start", c_void_p),
        ("cell_bucket", c_void_p),
        ("cell_rank", c_void_p),
        ("scatter", c_void_p),
        ("sorted_id", c_void_p),
        ("sorted_xyzr", c_void_p),
        ("scan_partials", c_void_p),
        ("capacity", c_int64),
    ]


class GridGeometryC(ctypes.Structure):
    _fields_ = [
        ("nx", c_int32),
        ("ny", c_int32),
        ("nz", c_int32),
        ("origin_x", c_float),
        ("origin_y", c_float),
        ("origin_z", c_float),
        ("inv_dx", c_float),
    ]


class TissueRegionC(ctypes.Structure):
    _fields_ = [
        ("geom", GridGeometryC),
        ("sdf", c_void_p),
        ("gradient", c_void_p),
        ("wall_rate", c_float),
    ]


class SorParamsC(ctypes.Structure):
    _fields_ = [
        ("nx", c_int32),
        ("ny", c_int32),
        ("nz", c_int32),
        ("bc_x", c_int32),
        ("bc_y", c_int32),
        ("bc_z", c_int32),
        ("omega", c_float),
        ("dx2_over_D", c_float),
        ("uptake_max", c_float),
        ("michaelis_k", c_float),
        ("reference", c_float),
        ("has_source", c_int32),
        ("source_k", c_float),
    ]


class SorReportC(ctypes.Structure):
    _fields_ = [
        ("sweeps", c_int32),
        ("residual", c_float),
        ("converged", c_int32),
        ("path", c_int32),
        ("tiles", c_int32),
        ("strips", c_int32),
    ]


class SorTuningC(ctypes.Structure):
    _fields_ = [
        ("tiles", c_int32),
        ("strips", c_int32),
    ]


class LifecycleParamsC(ctypes.Structure):
    _fields_ = [
        ("dt", c_float),
        ("death_rate", c_float),
        ("anoxic_death_rate", c_float),
        ("division_rate", c_float),
        ("inhibition_threshold", c_int32),
        ("hypoxia_threshold", c_float),
        ("death_threshold", c_float),
        ("glucose_threshold", c_float),
        ("glucose_death_threshold", c_float),
        ("necrosis_requires_glucose", c_int32),
        ("phenotype_model", c_int32),
        ("apoptosis_rate", c_float),
        ("necrosis_rate", c_float),
    ]


class BatchInstanceC(ctypes.Structure):
    _fields_ = [
        ("capacity", c_int32),
        ("position", c_void_p),
        ("radius", c_void_p),
        ("cell_state", c_void_p),
        ("cell_type", c_void_p),
        ("age", c_void_p),
        ("oxygen_local", c_void_p),
        ("glucose_local", c_void_p),
        ("rng_state", c_void_p),
        ("velocity", c_void_p),
        ("neighbor_count", c_void_p),
        ("divide_flag", c_void_p),
        ("division_offset", c_void_p),
        ("fate_flags", c_void_p),
        ("grid", NeighborGridC),
        ("query_radius", c_float),
        ("contact_rate", c_float),
        ("contact_dt", c_float),
        ("contact_substeps", c_int32),
        ("geom", GridGeometryC),
        ("accumulator", c_void_p),
        ("density", c_void_p),
        ("uptake_density", c_void_p),
        ("uptake_weights", c_float * 4),
        ("inv_voxel_volume", c_float),
        ("field", c_void_p),
        ("lifecycle", LifecycleParamsC),
        ("placement_factor", c_float),
    ]


class BatchC(ctypes.Structure):
    _fields_ = [
        ("instances", c_int32),
        ("device_plan", c_void_p),
        ("cell_chunks", c_int32),
        ("node_chunks", c_int32),
        ("bucket_tiles", c_int32),
        ("slot_tiles", c_int32),
        ("max_substeps", c_int32),
    ]


class SorBatchItemC(ctypes.Structure):
    _fields_ = [
        ("params", SorParamsC),
        ("fixed", c_void_p),
        ("density", c_void_p),
        ("production", c_void_p),
        ("source", c_void_p),
        ("field", c_void_p),
        ("workspace", c_void_p),
    ]


class SorBatchC(ctypes.Structure):
    _fields_ = [
        ("items", c_int32),
        ("total_tiles", c_int32),
        ("ctas", c_int32),
        ("threads", c_int32),
        ("zclamp", c_int32),
        ("has_prod", c_int32),
        ("smem_bytes", c_int64),
        ("device_plan", c_void_p),
    ]


class NetworkProgramC(ctypes.Structure):
    _fields_ = [
        ("n_nodes", c_int32),
        ("n_words", c_int32),
        ("n_ops", c_int32),
        ("n_updatable", c_int32),
        ("ops", c_void_p),
        ("args", c_void_p),
        ("start", c_void_p),
        ("length", c_void_p),
        ("updatable", c_void_p),
        ("table_arity", c_void_p),
        ("table_inputs", c_void_p),
        ("table_bits", c_void_p),
    ]


_P = c_void_p
_I = c_int32
_F = c_float
# name -> argtypes (every function returns int32 unless listed in _RESTYPE)
SIGNATURES: dict[str, list] = {
    "wbc_version": [],
    "wbc_last_error": [],
    "wbc_device_count": [],
    "wbc_launch_count": [],
    "wbc_scan_workspace_bytes": [c_int64],
    "wbc_rng_init": [_I, _P, c_int64, _P],
    "wbc_rng_uniform": [_I, _I, _P, _P, _P],
    "wbc_rng_sphere": [_I, _P, _P, _P],
    "wbc_expf_batch": [_I, _P, _P, _P],
    "wbc_div_batch": [_I, _P, _P, _P, _P],
    "wbc_div_check": [_I, _I, _I, ctypes.c_uint32, ctypes.c_int64, _P, _P, _P],
    "wbc_grid_build": [POINTER(NeighborGridC), _I, _P, _P, _P],
    "wbc_contact_substep": [POINTER(NeighborGridC), _I, _F, _F, _F, _P, _P, _P, _P],
    "wbc_deposit": [POINTER(GridGeometryC), _I, _P, _P, _P, _P],
    "wbc_density_convert": [c_int64, _P, _F, _P, _P, _P, _I, _P],
    "wbc_density_combine": [c_int64, _P, _P, _P, _P],
    "wbc_sample": [POINTER(GridGeometryC), _P, _I, _P, _P, _P],
    "wbc_sor_sweeps": [POINTER(SorParamsC), _I, _P, _P, _P, _P, _P, _P, _P],
    "wbc_ftcs_step": [POINTER(SorParamsC), _F, _P, _P, _P, _P, _P, _P, _P],
    "wbc_sor_solve_workspace_bytes": [POINTER(SorParamsC)],
    "wbc_sor_wait_selftest": [_I, _I, _I, _P, c_size_t, _P],
    "wbc_sor_solve": [POINTER(SorParamsC), _I, _I, ctypes.c_double, _P, _P, _P, _P, _P, _P, POINTER(SorReportC),
                      _P, c_size_t, _I, POINTER(SorTuningC), _P],
    "wbc_sor_report_record_bytes": [],
    "wbc_sor_solve_deferred": [POINTER(SorParamsC), _I, _I, ctypes.c_double, _P, _P, _P, _P, _P, _P, _P, _P,
                               c_size_t, _I, POINTER(SorTuningC), _P],
    "wbc_sor_report_decode": [_P, POINTER(SorReportC)],
    "wbc_sor_autotune": [POINTER(SorParamsC), _I, _P, _P, _P, _P, _P, _P, _P, c_size_t, POINTER(SorTuningC),
                         POINTER(c_float), _P],
    "wbc_sor_batch_plan_bytes": [_I],
    "wbc_sor_batch_plan_host": [_I, POINTER(SorParamsC), _P, _I, c_int64, _P, _P, _P, _P, _P],
    "wbc_sor_batch_prepare": [_I, POINTER(SorBatchItemC), _P, _I, _I, ctypes.c_double, _P, c_size_t,
                              POINTER(SorBatchC), _P],
    "wbc_sor_batch_solve": [POINTER(SorBatchC), _P],
    "wbc_sor_batch_reports": [POINTER(SorBatchC), POINTER(SorReportC), _P],
    "wbc_batch_plan_bytes": [_I, POINTER(BatchInstanceC)],
    "wbc_batch_prepare": [_I, POINTER(BatchInstanceC), _P, c_size_t, POINTER(BatchC), _P],
    "wbc_batch_grid_build": [POINTER(BatchC), _P, _P],
    "wbc_batch_contact": [POINTER(BatchC), _P, _P],
    "wbc_batch_deposit": [POINTER(BatchC), _P, _P],
    "wbc_batch_sample": [POINTER(BatchC), _P, _P],
    "wbc_batch_lifecycle": [POINTER(BatchC), _P, _P, _P],
    "wbc_deposit_weighted": [POINTER(GridGeometryC), _I, _P, _P, _P, _P],
    "wbc_weighted_convert": [c_int64, _P, _F, _P, _I, _P],
    "wbc_adjoint_contact": [POINTER(NeighborGridC), _I, _F, _F, _F, _P, _P, _P, _P],
    "wbc_adjoint_field_solve": [POINTER(SorParamsC), _P, _P, _P, _P, _P, _I, _I, _F, _P, _P, _P,
                                POINTER(SorReportC), _P],
    "wbc_adjoint_cells": [POINTER(GridGeometryC), _I, _P, _P, _P, _F, _P, _P, _P],
    "wbc_contact_steps_workspace_bytes": [_I, c_int64, _I],
    "wbc_deposit32_bytes": [c_int64],
    "wbc_deposit32": [POINTER(GridGeometryC), _I, _P, _P, _P, _P, c_size_t, _P],
    "wbc_convert32": [c_int64, _P, _F, _P, _P, _P, _P],
    "wbc_contact_steps": [POINTER(NeighborGridC), _I, _F, _F, _F, _I, _P, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _P,
                          c_size_t, _I, _P],
    "wbc_adjoint_steps": [POINTER(NeighborGridC), _I, _F, _F, _F, _I, _I, _P, _P, _P, _I, _P, c_size_t, _I, _P],
    "wbc_sor_linear_solve": [POINTER(SorParamsC), _I, _I, ctypes.c_double, _P, _P, _P, POINTER(SorReportC), _P,
                             c_size_t, _P],
    "wbc_adjoint_newton_prepare": [POINTER(SorParamsC), _P, _P, _P, _P, _P],
    "wbc_adjoint_newton_apply": [c_int64, _P, _P, _P],
    "wbc_widen": [c_int64, _P, _P, _P],
    "wbc_narrow": [c_int64, _P, _P, _P],
    "wbc_fill": [c_int64, c_float, _P, _P],
    "wbc_zero": [_P, c_size_t, _P],
    "wbc_divide": [c_int64, _P, c_float, _P, _P],
    "wbc_compensated_sum": [c_int64, _P, _P, _P, _P, _P],
    "wbc_mean": [c_int64, _P, _P, _P],
    "wbc_adjoint_linear_residual": [POINTER(SorParamsC), _P, _P, _P, _P, _P],
    "wbc_adjoint_field_grads": [POINTER(SorParamsC), _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "wbc_contact_substep_region": [POINTER(NeighborGridC), _I, _F, _F, _F, POINTER(TissueRegionC), _P, _P, _P, _P],
    "wbc_sample_sdf": [POINTER(TissueRegionC), _I, _P, _P, _P],
    "wbc_lifecycle_decide": [POINTER(LifecycleParamsC), _I, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "wbc_division_scan": [_I, _P, _P, _P, _P, c_size_t, _P],
    "wbc_division_scan_noalloc": [_I, _P, _P, _P, _P],
    "wbc_place_daughters": [_I, _F, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "wbc_count_states": [_I, _P, _P, _P],
    "wbc_network_initialize": [POINTER(NetworkProgramC), _I, _P, _P, _P, _P],
    "wbc_network_clamp_inputs": [_I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "wbc_network_update_sync": [POINTER(NetworkProgramC), _I, _I, _P, _P],
    "wbc_network_update_async": [POINTER(NetworkProgramC), _I, _I, _P, _P, _P],
    "wbc_network_update_maboss": [POINTER(NetworkProgramC), _I, _F, _I, _P, _P, _P, _P, _P, _P, _P],
    "wbc_network_read_fates": [_I, _I, _I, _I, _I, _I, _P, _P, _P],
    "wbc_network_inherit": [_I, _I, _P, _P, _P, _P],
    "wbc_network_count_on": [_I, _I, _I, _P, _I, _P, _P, _P, _P],
}
_RESTYPE = {"wbc_last_error": ctypes.c_char_p, "wbc_scan_workspace_bytes": c_size_t, "wbc_launch_count": c_int64,
            "wbc_sor_solve_workspace_bytes": c_size_t, "wbc_sor_batch_plan_bytes": c_size_t,
            "wbc_batch_plan_bytes": c_size_t, "wbc_contact_steps_workspace_bytes": c_size_t,
            "wbc_deposit32_bytes": c_size_t, "wbc_sor_report_record_bytes": c_size_t}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def load(path: str | Path | None = None) -> ctypes.CDLL:
    """Load the library once (raises LibraryError when it was not built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else library_path()
        if not p.exists():
            raise LibraryError(
                f"{p} is missing: build the native library first (python -c 'import __graft_entry__ as g; g.build()')"
            )
        try:
            lib = ctypes.CDLL(str(p))
        except OSError as exc:
            raise LibraryError(f"cannot load {p}: {exc}") from exc
        for name, argtypes in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = _RESTYPE.get(name, c_int32)
        _lib = lib
        return lib


def launch_count() -> int:
    """Kernels launched by libwbc_gb300 in this process so far."""
    return int(load().wbc_launch_count())


def last_error() -> str:
    return load().wbc_last_error().decode(errors="replace")


def check(rc: int, what: str) -> None:
    if rc == WBC_OK:
        return
    if rc == WBC_ERR_CUDA:
        raise LibraryError(f"{what}: CUDA error: {last_error()}")
    if rc == WBC_ERR_WORKSPACE:
        raise LibraryError(f"{what}: workspace too small")
    if rc == WBC_ERR_TIMEOUT:
        raise LibraryError(f"{what}: a device-side wait timed out")
    raise ValueError(f"{what}: invalid arguments (status {rc}): {last_error()}")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


def ptr(t: torch.Tensor | None) -> int | None:
    """Device pointer of a contiguous CUDA tensor (None stays NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise RuntimeError("warpbiocell_gb300 arrays live on a CUDA device; got a CPU tensor (there is no CPU fallback)")
    if not t.is_contiguous():
        raise ValueError("arrays passed to the native library must be contiguous")
    return t.data_ptr()


def stream(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def resolve_device(device=None) -> torch.device:
    """CUDA device for a drop-in ``device`` argument: None/'auto'/'cuda'/'cuda:N'/torch.device.

    'cpu' is rejected: the reference's Warp CPU path has no counterpart here by design.
    """
    if isinstance(device, torch.device):
        dev = device
    elif device is None or device == "auto":
        dev = torch.device("cuda", torch.cuda.current_device() if torch.cuda.is_available() else 0)
    else:
        dev = torch.device(str(device))
    if dev.type != "cuda":
        raise RuntimeError(f"device {device!r}: warpbiocell_gb300 runs on CUDA devices only (no CPU fallback)")
    if not torch.cuda.is_available():
        raise RuntimeError("no CUDA device is available: warpbiocell_gb300 needs a GPU")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    load()
    return dev

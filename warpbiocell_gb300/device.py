"""Device selection (reference: device.py).

The same three calls as the reference's module. Devices are ``torch.device`` objects and are
always CUDA devices: ``"auto"`` (or None) picks the current CUDA device, and ``"cpu"`` is refused,
because the reference's Warp CPU path has no counterpart in this package.
"""

from __future__ import annotations

import torch

from warpbiocell_gb300 import _lib


def resolve_device(name: str | None = "auto") -> torch.device:
    """The CUDA device named by ``name`` (None, ``"auto"``, ``"cuda"``, ``"cuda:N"`` or a
    ``torch.device``); raises RuntimeError for ``"cpu"`` or when no GPU is present."""
    return _lib.resolve_device(name)


def cuda_available() -> bool:
    return torch.cuda.is_available()


def synchronize(device) -> None:
    """Block until all work queued on ``device`` has finished."""
    dev = device if isinstance(device, torch.device) else torch.device(str(device))
    if dev.type == "cuda":
        torch.cuda.synchronize(dev)

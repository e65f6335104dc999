"""Optional per-stage device timing with CUDA events.

When enabled, each hot-path call records a start and an end event on the torch stream it
launches on (the same stream the kernels run on), so stage durations are device time, not host
time. Disabled by default: ``stage(...)`` is then a no-op context manager. The benchmark enables
it around its timed region to attribute the step time to binning, contact, deposit, SOR,
sample, lifecycle and scan/placement.
"""

from __future__ import annotations

from collections import defaultdict
from contextlib import contextmanager

import torch

_enabled = False
_only: frozenset[str] | None = None
_events: list[tuple[str, torch.cuda.Event, torch.cuda.Event, int]] = []


def enable(on: bool = True, only=None) -> None:
    """Start (or stop) recording; ``only``: the stage names to time (default every stage)."""
    global _enabled, _only
    _enabled = on
    _only = frozenset(only) if only is not None else None
    _events.clear()


def enabled() -> bool:
    return _enabled


@contextmanager
def stage(name: str, launches: int = 1):
    """Time the enclosed launches as stage ``name`` (``launches`` kernels are attributed to it)."""
    if not _enabled or (_only is not None and name not in _only):
        yield
        return
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record()
    try:
        yield
    finally:
        end.record()
        _events.append((name, start, end, launches))


def summary() -> dict[str, dict[str, float]]:
    """{stage: {"ms": total device ms, "calls": n, "launches": kernels}} (synchronises)."""
    torch.cuda.synchronize()
    out: dict[str, dict[str, float]] = defaultdict(lambda: {"ms": 0.0, "calls": 0, "launches": 0})
    for name, start, end, launches in _events:
        s = out[name]
        s["ms"] += start.elapsed_time(end)
        s["calls"] += 1
        s["launches"] += launches
    return dict(out)

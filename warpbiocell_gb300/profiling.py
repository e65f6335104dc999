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
_events: list[tuple[str, torch.cuda.Event, torch.cuda.Event, int]] = []


def enable(on: bool = True) -> None:
    global _enabled
    _enabled = on
    _events.clear()


def enabled() -> bool:
    return _enabled


@contextmanager
def stage(name: str, launches: int = 1):
    """Time the enclosed launches as stage ``name`` (``launches`` kernels are attributed to it)."""
    if not _enabled:
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

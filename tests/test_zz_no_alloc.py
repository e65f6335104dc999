"""The allocation-free division scan against the workspace one, through the C-ABI.

Some callers cannot allocate device memory (their host framework owns the device memory budget,
or their loop must not take the device-wide synchronisation cudaMalloc can cause), so the
library offers wbc_division_scan_noalloc, whose scratch lives in a fixed array inside the
library. This file is collected last on purpose: if it fails, a run that stops at the first
failure has already run every other test. It must pass alone in a fresh process too.
"""

import numpy as np
import pytest
import torch

from warpbiocell_gb300 import _lib

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _scan_with_workspace(flags: torch.Tensor):
    lib = _lib.load()
    n = flags.numel()
    out = torch.full_like(flags, -7)
    total = torch.full((1,), -7, dtype=torch.int32, device=DEV)
    nbytes = int(lib.wbc_scan_workspace_bytes(max(n, 1)))
    ws = torch.empty((nbytes + 3) // 4, dtype=torch.int32, device=DEV)
    _lib.check(lib.wbc_division_scan(n, _lib.ptr(flags), _lib.ptr(out), _lib.ptr(total), _lib.ptr(ws), nbytes,
                                     _lib.stream(torch.device(DEV))), "wbc_division_scan")
    return out, total


def _scan_no_alloc(flags: torch.Tensor):
    lib = _lib.load()
    out = torch.full_like(flags, -7)
    total = torch.full((1,), -7, dtype=torch.int32, device=DEV)
    _lib.check(lib.wbc_division_scan_noalloc(flags.numel(), _lib.ptr(flags), _lib.ptr(out), _lib.ptr(total),
                                             _lib.stream(torch.device(DEV))), "wbc_division_scan_noalloc")
    return out, total


def test_no_alloc_scan_matches_workspace_scan_on_two_calls_in_a_row():
    rng = np.random.default_rng(2024)
    # a large call then a smaller one: the second must not see the first call's partials
    for n, p in ((3_000_001, 0.3), (70_001, 0.7)):
        flags = torch.as_tensor((rng.random(n) < p).astype(np.int32), device=DEV)
        ref, ref_total = _scan_with_workspace(flags)
        got, got_total = _scan_no_alloc(flags)
        torch.cuda.synchronize()
        assert torch.equal(got, ref)
        assert int(got_total.item()) == int(ref_total.item()) == int(flags.sum().item())


def test_no_alloc_scan_of_no_cells_writes_a_zero_total():
    # n = 0 launches nothing and only sets the total, as the workspace scan does
    empty = torch.zeros(0, dtype=torch.int32, device=DEV)
    ref, ref_total = _scan_with_workspace(empty)
    got, got_total = _scan_no_alloc(empty)
    torch.cuda.synchronize()
    assert got.numel() == ref.numel() == 0
    assert int(got_total.item()) == int(ref_total.item()) == 0


def test_no_alloc_scan_at_its_exact_limit():
    # WBC_NOALLOC_SCAN_MAX_CELLS cells fill every tile partial, the total's entry included
    n = 33_554_432
    rng = np.random.default_rng(7)
    flags = torch.zeros(n, dtype=torch.int32, device=DEV)
    hits = torch.as_tensor(rng.choice(n, size=50_000, replace=False), device=DEV)
    flags[hits] = 1
    flags[-1] = 1  # the last cell divides: its offset is the total
    ref, ref_total = _scan_with_workspace(flags)
    got, got_total = _scan_no_alloc(flags)
    torch.cuda.synchronize()
    assert torch.equal(got, ref)
    assert int(got_total.item()) == int(ref_total.item()) == int(flags.sum().item())
    assert int(got[-1].item()) == int(got_total.item())
    del flags, ref, got


def test_no_alloc_scan_rejects_sizes_beyond_its_limit():
    lib = _lib.load()
    dummy = torch.zeros(1, dtype=torch.int32, device=DEV)
    rc = lib.wbc_division_scan_noalloc(33554433, _lib.ptr(dummy), _lib.ptr(dummy), None,
                                       _lib.stream(torch.device(DEV)))
    assert rc == _lib.WBC_ERR_INVALID
    assert "WBC_NOALLOC_SCAN_MAX_CELLS" in _lib.last_error()

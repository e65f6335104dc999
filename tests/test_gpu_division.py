"""The solver's correctly rounded division (Markstein's FMA method over the hardware reciprocal
estimate) against IEEE division: the refined reciprocal exhaustively over every float the fast path
accepts, seeded operand pairs of every class on the device, and a batch against numpy's float32
division on the host."""

import numpy as np
import pytest
import torch

from warpbiocell_gb300 import _lib

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _check(mode, e_lo=0, e_hi=0, seed=0, pairs=0):
    count = torch.zeros(1, dtype=torch.int64, device=DEV)
    first = torch.zeros(2, dtype=torch.int32, device=DEV)
    _lib.call("wbc_div_check", mode, e_lo, e_hi, seed, pairs, _lib.ptr(count), _lib.ptr(first), _lib.stream(DEV))
    torch.cuda.synchronize()
    bad = first.cpu().numpy().view(np.uint32)
    return int(count.item()), bad.view(np.float32)


def test_refined_reciprocal_is_correctly_rounded_for_every_fast_path_divisor():
    count, bad = _check(0, -60, 60)
    assert count == 0, f"{count} reciprocals differ, first b = {bad[1]!r}"


@pytest.mark.parametrize("seed", [1, 2])
def test_division_matches_ieee_on_seeded_pairs(seed):
    count, bad = _check(1, seed=seed, pairs=1 << 30)
    assert count == 0, f"{count} quotients differ, first a/b = {bad[0]!r}/{bad[1]!r}"


def test_division_batch_matches_numpy():
    rng = np.random.default_rng(5)
    n = 1 << 20
    a = rng.standard_normal(n).astype(np.float32) * np.exp2(rng.integers(-70, 70, n)).astype(np.float32)
    b = rng.standard_normal(n).astype(np.float32) * np.exp2(rng.integers(-70, 70, n)).astype(np.float32)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 3e38, 1e-38, 1.0], np.float32)
    a[: special.size * special.size] = np.repeat(special, special.size)
    b[: special.size * special.size] = np.tile(special, special.size)
    out = torch.empty(n, dtype=torch.float32, device=DEV)
    ta, tb = torch.from_numpy(a).to(DEV), torch.from_numpy(b).to(DEV)
    _lib.call("wbc_div_batch", n, _lib.ptr(ta), _lib.ptr(tb), _lib.ptr(out), _lib.stream(DEV))
    with np.errstate(all="ignore"):
        want = a / b
    got = out.cpu().numpy()
    nan = np.isnan(want)
    np.testing.assert_array_equal(np.isnan(got), nan)
    np.testing.assert_array_equal(got[~nan].view(np.uint32), want[~nan].view(np.uint32))

"""The batched solve's planner (wbc_sor_batch_plan_host: the plan wbc_sor_batch_prepare makes,
computed on the host): every member placed once, members ordered by sweep count, waves that fit
on the GPU, compact tilings, equal-finish tile counts, and the planner's own objective no worse
than simple plans. Host code only; no GPU."""

import ctypes

import numpy as np
import pytest

CTAS = 152
SMEM = 232448 - 1024  # the GB300's opt-in shared memory per block, less the static part

# the benchmark's 15-spheroid sweep: grid sides and the sweep counts of a late step
SIDES = [55, 93, 79, 71, 69, 105, 113, 55, 93, 65, 119, 115, 91, 101, 83]
SWEEPS = [140, 160, 160, 220, 240, 140, 200, 120, 280, 200, 280, 280, 340, 500, 240]


@pytest.fixture(scope="module")
def lib():
    from warpbiocell_gb300 import _build, _lib

    if not _build.library_path().exists():
        _build.build()
    return _lib.load()


def plan(lib, sides, sweeps=None, ctas=CTAS, smem=SMEM):
    from warpbiocell_gb300 import _lib

    n = len(sides)
    params = (_lib.SorParamsC * n)()
    for k, s in enumerate(sides):
        params[k].nx = params[k].ny = params[k].nz = s
    weights = None
    if sweeps is not None:
        weights = (ctypes.c_float * n)(*[float(s) ** 3 * w for s, w in zip(sides, sweeps)])
    order, tiles, strips, wave = (np.zeros(n, np.int32) for _ in range(4))
    ns = np.zeros(n, np.float64)
    rc = lib.wbc_sor_batch_plan_host(n, params, weights, ctas, ctypes.c_int64(smem), order.ctypes.data,
                                     tiles.ctypes.data, strips.ctypes.data, wave.ctypes.data, ns.ctypes.data)
    return rc, order, tiles, strips, wave, ns


def test_every_member_is_planned_once_in_waves_that_fit(lib):
    rc, order, tiles, strips, wave, ns = plan(lib, SIDES, SWEEPS)
    assert rc == 0
    assert sorted(order.tolist()) == list(range(len(SIDES)))
    assert (tiles >= 1).all() and (strips >= 1).all() and (strips <= tiles).all()
    assert (np.diff(wave) >= 0).all() and wave[0] == 0  # waves are contiguous runs of the work list
    for w in range(wave.max() + 1):
        assert tiles[wave == w].sum() <= CTAS, w
    # members ordered by sweep count, most first
    sw = np.array(SWEEPS)[order]
    assert (np.diff(sw) <= 0).all()


def test_a_wave_ends_together(lib):
    """Within a wave no member could finish sooner without the wave needing more CTAs than the
    GPU has: the slowest member's modelled duration bounds every other's."""
    rc, order, tiles, strips, wave, ns = plan(lib, SIDES, SWEEPS)
    dur = np.array(SWEEPS)[order] * ns
    for w in range(wave.max() + 1):
        d = dur[wave == w]
        assert d.max() > 0
        # the members of a wave are sized to the wave's duration: none runs below half of it
        # unless held at its fewest tiles
        held = tiles[wave == w] <= 2
        assert ((d >= 0.5 * d.max()) | held).all(), (w, d)


def test_tilings_are_compact(lib):
    """Strip counts near the square shape: no member runs on long thin tiles."""
    rc, order, tiles, strips, wave, ns = plan(lib, SIDES, SWEEPS)
    square = np.sqrt(tiles)
    assert (strips >= np.maximum(1, np.floor(square / 2))).all()
    assert (strips <= 2 * square + 2).all()


def test_the_dynamic_programme_beats_one_wave_per_member(lib):
    """The planner's objective (sum of its waves' modelled durations) is no worse than running
    the members one at a time on all CTAs."""
    rc, order, tiles, strips, wave, ns = plan(lib, SIDES, SWEEPS)
    dur = np.array(SWEEPS)[order] * ns
    planned = sum(dur[wave == w].max() for w in range(wave.max() + 1))
    alone = 0.0
    for s, sw in zip(SIDES, SWEEPS):
        rc1, _, _, _, _, ns1 = plan(lib, [s], [sw])
        assert rc1 == 0
        alone += sw * ns1[0]
    assert planned < alone


def test_without_weights_members_are_ordered_by_size(lib):
    rc, order, tiles, strips, wave, ns = plan(lib, SIDES)
    assert rc == 0
    sizes = np.array(SIDES)[order]
    assert (np.diff(sizes) <= 0).all()


def test_the_plan_is_deterministic(lib):
    a = plan(lib, SIDES, SWEEPS)
    b = plan(lib, SIDES, SWEEPS)
    for x, y in zip(a[1:], b[1:]):
        np.testing.assert_array_equal(x, y)


def test_a_grid_larger_than_shared_memory_is_refused(lib):
    rc = plan(lib, [55, 400])[0]
    assert rc == -1
    assert b"does not fit" in lib.wbc_last_error()


def test_bad_arguments_are_refused_before_planning(lib):
    assert plan(lib, [55], ctas=0)[0] == -1
    assert plan(lib, [2])[0] == -1
    assert plan(lib, [55], [0.0])[0] == -1

"""The baked-to-live hand-off (ADR-0080 decision 4): a tile starts from the baked answer and retires
to it when its state has settled back within a stated bound. The start is wl_batch_write_tile_state
between ticks or a WL_EVENT_STATE through the tick queue (test_queue_gpu.py); the check is
wl_settled / wl_batch_settled: per tile the largest |h - h*| and the largest of |hu - hu*| and
|hv - hv*| against the steady state rounded to f32, held here to numpy's f32 arithmetic on the
state read back, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

import cases
from pairs import make_pair

pytestmark = pytest.mark.gpu


def deviations(planes, h, hu, hv):
    """numpy's statement of the check: f32 differences (correctly rounded), their largest."""
    n = h.size
    st = planes.reshape(4, n)
    f = lambda a: np.asarray(a, np.float64).astype(np.float32)
    dd = np.max(np.abs(st[0] - f(h)))
    dq = max(np.max(np.abs(st[1] - f(hu))), np.max(np.abs(st[2] - f(hv))))
    return np.float32(dd), np.float32(dq)


def test_a_lake_at_rest_is_settled_and_a_sloshing_basin_is_not(gpu):
    c = cases.exact_lake()
    dev, _ = make_pair(c)
    n = c["nx"] * c["ny"]
    z = np.zeros(n)
    ok, dd, dq = dev.settled(c["h"], z, z, 0.0, 0.0)
    assert ok and dd == 0.0 and dq == 0.0  # the lake at rest is its own baked answer
    assert dev.run_steps(40, 0.02), dev.error
    ok, dd, dq = dev.settled(c["h"], z, z, 0.0, 0.0)
    assert ok and dd == 0.0 and dq == 0.0  # and stays so, exactly (well-balanced)

    b = cases.closed_basin()
    dev, _ = make_pair(b)
    n = b["nx"] * b["ny"]
    level = np.maximum(0.4 - np.asarray(b["bed"]), 0.0)  # a made-up steady answer
    z = np.zeros(n)
    for ticks in (0, 25, 100):
        if ticks:
            assert dev.run_steps(ticks, 0.01), dev.error
        want_dd, want_dq = deviations(dev.read_state_bits(), level, z, z)
        ok, dd, dq = dev.settled(level, z, z, 0.05, 0.01)
        assert (np.float32(dd), np.float32(dq)) == (want_dd, want_dq), ticks
        assert ok == bool(want_dd <= np.float32(0.05) and want_dq <= np.float32(0.01))
        ok_loose, _, _ = dev.settled(level, z, z, float(want_dd), float(want_dq))
        assert ok_loose  # the bounds are inclusive
    assert not dev.settled(level[:-1], z[:-1], z[:-1], 1.0, 1.0)  # misfit: refused
    assert dev.last_code == 2


def test_a_batch_reports_each_tile(gpu):
    from game_engine_gb300.batch import Batch
    from test_batch_gpu import load, mixed_tiles
    tiles, sides, edges = mixed_tiles()
    b = Batch(sides, open_edges=edges)
    load(b, tiles)
    b.run_ticks(30, 0.02)
    steady = [np.maximum(1.9 - np.asarray(t.bed), 0.0) for t in tiles]
    h = np.concatenate(steady)
    z = np.zeros_like(h)
    ok, dd, dq = b.settled(h, z, z, 0.3, 0.05)
    for k, t in enumerate(tiles):
        want_dd, want_dq = deviations(b.read_tile_bits(k), steady[k], np.zeros(t.cells),
                                      np.zeros(t.cells))
        assert (dd[k], dq[k]) == (want_dd, want_dq), k
        assert ok[k] == bool(want_dd <= np.float32(0.3) and want_dq <= np.float32(0.05))
    b.close()


def test_wake_step_and_retire_a_tile(gpu):
    """The hand-off's round trip on one tile of a batch: it wakes from its baked answer, is
    disturbed by a source and steps, so it has not settled; it retires (its state written back to
    the baked answer), after which it checks settled with no deviation, and the retiring write
    leaves the other tiles as they were."""
    from game_engine_gb300.batch import Batch
    from test_batch_gpu import mixed_tiles
    tiles, sides, edges = mixed_tiles()
    b = Batch(sides, open_edges=[0] * len(sides))
    b.set_bed(np.concatenate([t.bed for t in tiles]))
    baked = [np.maximum(1.2 - np.asarray(t.bed), 0.0) for t in tiles]
    b.write_state(np.concatenate(baked))
    k = 7  # 64 x 130
    n = tiles[k].cells
    z = np.zeros(n)
    src = np.zeros(b.cells)
    sl = b.tile_slice(k)
    src[sl] = np.where(np.arange(n) % 97 == 0, 2e-3, 0.0)
    b.set_source(src)
    b.run_ticks(20, 0.02)
    ok, dd, _ = b.settled(np.concatenate(baked), np.zeros(b.cells), np.zeros(b.cells), 1e-4, 1e-4)
    assert not ok[k] and dd[k] > 0.0
    b.set_source(None)
    others = [b.read_tile_bits(j) for j in range(len(tiles)) if j != k]
    b.write_tile_state(k, baked[k], z, z)  # retire: the baked answer back
    ok, dd, dq = b.settled(np.concatenate(baked), np.zeros(b.cells), np.zeros(b.cells), 0.0, 0.0)
    assert ok[k] and dd[k] == 0.0 and dq[k] == 0.0
    rest = [b.read_tile_bits(j) for j in range(len(tiles)) if j != k]
    for a, c in zip(others, rest):  # the retiring write touches its own tile alone
        assert np.array_equal(a.view(np.uint32), c.view(np.uint32))
    b.close()

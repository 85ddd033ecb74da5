"""The three-phase block tick's staged variant: each 32 x 16 block's cells and one-cell halo taken
into shared memory by two tensor copies (TMA) in place of each thread's loads, for tiles whose width
is a multiple of 4. By default it runs where 256-thread block CTAs step blocks in turn, each CTA's
next block's copies landing while it steps the last; WLCUDA_STAGE=1 turns it on in every block
launch. Held to the oracle bit for bit: a launch a tick on every case and flag, both forms of the
arithmetic; batches of uneven tiles (widths that take the copies beside widths that load cell by
cell) in the 512-thread CTA (no more blocks than SMs) and the 256-thread one (many blocks a CTA);
the tick queue, whose landed tiles skip their blocks."""
from __future__ import annotations

import os
from contextlib import contextmanager

import numpy as np
import pytest

import cases
from pairs import assert_same, make_pair

pytestmark = pytest.mark.gpu


@contextmanager
def staged():
    """Steps created inside take the staged variant (WLCUDA_STAGE=1)."""
    old = os.environ.get("WLCUDA_STAGE")
    os.environ["WLCUDA_STAGE"] = "1"
    try:
        yield
    finally:
        if old is None:
            os.environ.pop("WLCUDA_STAGE", None)
        else:
            os.environ["WLCUDA_STAGE"] = old


def lake_256():
    from game_engine_gb300 import workloads
    t = workloads.plain_256()
    return dict(nx=t.nx, ny=t.ny, cell_m=t.cell_m, bed=t.bed, h=t.h, source=t.source)


CASES = {
    "slope": lambda: cases.slope(),  # Manning's n, a source, an open edge
    "slope_all_open": lambda: cases.slope(all_open=True),
    "closed_basin": cases.closed_basin,
    "exact_lake": cases.exact_lake,
    "lake_256": lake_256,
}


def narrow():
    """32 x 20: narrower than a copy's box (40 columns) and shorter than it (18 rows), so every
    box reaches past the tile on both sides."""
    n = 32 * 20
    x, y = np.arange(n) % 32, np.arange(n) // 32
    return dict(nx=32, ny=20, cell_m=0.5, bed=0.01 * x + 0.02 * (y % 3),
                h=np.where(x < 10, 0.5, 0.05), open_edges=6)


SMALL = {"narrow": narrow, "dam_1d": lambda: cases.dam(400, 0.001)}


@pytest.mark.parametrize("name", sorted(SMALL))
def test_staged_tiles_smaller_than_a_box(gpu, name):
    """Tiles smaller than a copy's box: where the driver's encoder gives them tensor maps, the
    copies' cells past the tile arrive as zeros and are not read; either way, the oracle's bytes."""
    c = SMALL[name]()
    with staged():
        dev, ref = make_pair(c, rows=1)
    assert dev.staged_tiles() in (0, 1)
    print(f"{name}: staged_tiles {dev.staged_tiles()}")
    for _ in range(29):
        assert dev.run_steps(1, 0.01), dev.error
    ref.run_steps(29, 0.01)
    assert_same(dev, ref, name)
    dev.destroy()


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("fixed", [False, True])
def test_staged_launch_a_tick_equals_the_oracle(gpu, name, fixed):
    c = CASES[name]()
    with staged():
        dev, ref = make_pair(c, fixed=fixed, rows=1)
    assert dev.staged_tiles() == 1
    ticks, max_dt = 41, 0.02
    for _ in range(ticks):  # one tick a call: a launch a tick, not the resident tick
        assert dev.run_steps(1, max_dt), dev.error
    ref.run_steps(ticks, max_dt)
    assert_same(dev, ref, name)
    dev.destroy()


@pytest.mark.parametrize("every,compensate", [(1, True), (3, False), (4, True)])
def test_staged_source_clocks(gpu, every, compensate):
    c = cases.slope()
    with staged():
        dev, ref = make_pair(c, every=every, compensate=compensate, rows=1)
    assert dev.staged_tiles() == 1
    for _ in range(23):
        assert dev.run_steps(1, 0.05), dev.error
    ref.run_steps(23, 0.05)
    assert_same(dev, ref, f"every {every}, compensate {compensate}")
    dev.destroy()


@contextmanager
def stage_env(value):
    old = os.environ.get("WLCUDA_STAGE")
    if value is None:
        os.environ.pop("WLCUDA_STAGE", None)
    else:
        os.environ["WLCUDA_STAGE"] = value
    try:
        yield
    finally:
        if old is None:
            os.environ.pop("WLCUDA_STAGE", None)
        else:
            os.environ["WLCUDA_STAGE"] = old


@pytest.mark.parametrize("env,want", [(None, 1), ("0", 0)])
def test_the_default_stages_blocks_a_cta_steps_in_turn(gpu, env, want):
    """A 1024 x 512 tile (1024 blocks, more than the device's 256-thread CTAs: each CTA steps
    blocks in turn, the next one's copies landing while it steps the last) stages by default and
    not with WLCUDA_STAGE=0. A 512 x 512 tile (512 blocks, a CTA each) and a 256 x 256 one (128
    blocks: the 512-thread CTA) do not by default. The staged tile steps to the oracle's bytes."""
    nx, ny = 1024, 512
    n = nx * ny
    x, y = np.arange(n) % nx, np.arange(n) // nx
    c = dict(nx=nx, ny=ny, cell_m=0.5, bed=0.002 * x + 0.001 * (y % 7),
             h=np.where((x - 500) ** 2 + (y - 250) ** 2 < 2500, 1.2, 0.05))
    with stage_env(env):
        dev, ref = make_pair(c, rows=1)
        others = [make_pair(lake_256(), rows=1)[0],
                  make_pair(dict(nx=512, ny=512, cell_m=0.5, bed=np.zeros(512 * 512),
                                 h=np.full(512 * 512, 0.3)), rows=1)[0]]
    assert dev.staged_tiles() == want
    for o in others:
        assert o.staged_tiles() == 0
        o.destroy()
    for _ in range(12):
        assert dev.run_steps(1, 0.02), dev.error
    ref.run_steps(12, 0.02)
    assert_same(dev, ref, f"{nx} x {ny}, WLCUDA_STAGE={env}")
    dev.destroy()


def test_a_width_off_the_copy_boundary_loads_cell_by_cell(gpu):
    """A tile 50 wide (rows off 16-byte boundaries) takes no tensor maps and steps by loads."""
    n = 50 * 30
    x = np.arange(n) % 50
    c = dict(nx=50, ny=30, cell_m=0.5, bed=0.01 * x, h=np.where(x < 20, 0.6, 0.1))
    with staged():
        dev, ref = make_pair(c, rows=1)
    assert dev.staged_tiles() == 0
    for _ in range(17):
        assert dev.run_steps(1, 0.02), dev.error
    ref.run_steps(17, 0.02)
    assert_same(dev, ref, "50 wide")
    dev.destroy()


@pytest.mark.parametrize("graph", [True, False])
def test_staged_mixed_tiles_equal_their_oracles(gpu, graph):
    """Eight uneven tiles (four widths take the copies, four load cell by cell), open edges and a
    source, in no more blocks than SMs: the 512-thread CTA."""
    from test_batch_gpu import load, mixed_tiles, oracle_tile
    from game_engine_gb300.batch import Batch
    tiles, sides, edges = mixed_tiles()
    b = Batch(sides, open_edges=edges)
    b.set_tuning(1, 0, stage=1)
    assert b.tuning()["stage"] == 1
    assert b.staged_tiles() == sum(1 for nx, _ in sides if nx % 4 == 0) > 0
    load(b, tiles)
    b.run_ticks(37, 0.02, graph=graph)
    for k, t in enumerate(tiles):
        r = oracle_tile(t, edges[k], 37, 0.02)
        got = b.read_tile_bits(k)
        assert np.array_equal(got.view(np.uint32), r.read_state_bits().view(np.uint32)), \
            f"tile {k} {sides[k]}"
    b.close()


def test_staged_many_blocks_a_cta(gpu):
    """The batched configuration's tiles (dry land, a column each), more blocks than SMs: the
    256-thread CTA steps many blocks in turn, each next block's copies issued once the last
    block's reads of the stage are done. Every tile equals the unstaged blocks' bytes after 120
    ticks, and sampled tiles the oracle's."""
    from test_batch_gpu import load, oracle_tile
    from game_engine_gb300 import workloads
    from game_engine_gb300.batch import Batch
    tiles = workloads.tiles_4096(24)
    sides = [(t.nx, t.ny) for t in tiles]
    out = []
    for stage in (0, 1):
        b = Batch(sides)
        b.set_tuning(1, 1, stage=stage)
        if stage:
            assert b.staged_tiles() == sum(1 for nx, _ in sides if nx % 4 == 0) > 0
        load(b, tiles, source=False)
        b.run_ticks(120, 0.01)
        out.append(b.tile_hashes())
        b.close()
    assert np.array_equal(out[0], out[1])
    for k in (0, 11, 23):
        r = oracle_tile(tiles[k], 0, 120, 0.01, source=False)
        assert int(out[1][k]) == r.state_hash(), f"tile {k} {sides[k]}"


@pytest.mark.parametrize("case", ["slope", "basin"])
def test_staged_queue_equals_advance_per_tick(gpu, case):
    """The tick queue's slots on a staged step (a launch a slot, the queue's word letting it step;
    bed, source and Manning events between ticks) land where the oracle's advance-per-tick does."""
    from game_engine_gb300.tick_queue import TickQueue
    from test_queue_gpu import assert_same_after_ticks, device_run, oracle_run, plan_for
    c = cases.slope(False) if case == "slope" else cases.closed_basin()
    with staged():
        dev, ref = make_pair(c)
    assert dev.staged_tiles() == 1
    n = 18
    plan = plan_for(c, n, seed=5)
    want = oracle_run(ref, c, plan)
    q = TickQueue(dev, records=32, arena_values=4096, max_events=64)
    for tick, length, events in plan:
        assert q.push(tick, length, events), q.error
    device_run(q, n, [3, 1, 7])
    assert_same_after_ticks(dev, ref, f"staged queue {case}")
    assert [r["substeps"] for r in q.landed(0, n)] == want
    q.close()
    dev.destroy()

"""The batched form: many tiles of uneven sizes in one persistent launch per tick, held tile by
tile to the oracle bit for bit, to the per-tile-launch form, across every block shape and item
order the autotuner chooses among, with and without the captured graph.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from game_engine_gb300 import workloads
from game_engine_gb300.batch import Batch, concat

pytestmark = pytest.mark.gpu


def mixed_tiles():
    """Odd and even sizes, partial work items, open and closed edges, dry and wet."""
    sides = [(64, 64), (17, 33), (96, 96), (1, 50), (33, 200), (128, 40), (5, 5), (64, 130)]
    edges = [0, 5, 2, 15, 0, 8, 3, 0]
    tiles = []
    for k, (nx, ny) in enumerate(sides):
        x, y = np.meshgrid(np.arange(nx), np.arange(ny))
        bed = workloads.fbm(nx, ny, 3.0, 1000 + k)
        h = np.maximum(2.0 - bed, 0.0) + ((x // 4 + y // 4) % 5 == 0).ravel() * 0.4
        tiles.append(workloads.Tile(nx, ny, bed, h, source=np.full(nx * ny, 2e-4 * (k % 3 - 1))))
    return tiles, sides, edges


def load(b, tiles, source=True):
    b.set_bed(concat(tiles, "bed"))
    if source:
        b.set_source(concat(tiles, "source"))
    b.write_state(concat(tiles, "h"), concat(tiles, "hu"), concat(tiles, "hv"))


def oracle_tile(t, edges, ticks, max_dt, source=True):
    r = oracle.RefStep(oracle.Grid(t.nx, t.ny, t.cell_m, open_edges=edges))
    r.set_bed(t.bed)
    if source:
        r.set_source(t.source)
    r.write_state(t.h, t.hu, t.hv)
    r.run_steps(ticks, max_dt)
    return r


@pytest.mark.parametrize("graph", [True, False])
def test_each_tile_equals_its_oracle(gpu, graph):
    tiles, sides, edges = mixed_tiles()
    b = Batch(sides, open_edges=edges)
    load(b, tiles)
    b.run_ticks(37, 0.02, graph=graph)
    hashes = b.tile_hashes()
    ledgers = b.ledgers()
    for k, t in enumerate(tiles):
        r = oracle_tile(t, edges[k], 37, 0.02)
        want = r.read_state_bits()
        got = b.read_tile_bits(k)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"tile {k} {sides[k]}"
        assert int(hashes[k]) == r.state_hash()
        assert ledgers[k] == r.read_ledger(), f"tile {k} ledger"


def test_per_tile_launches_give_the_same_bytes(gpu):
    tiles, sides, edges = mixed_tiles()
    a = Batch(sides, open_edges=edges)
    c = Batch(sides, open_edges=edges)
    load(a, tiles)
    load(c, tiles)
    a.run_ticks(25, 0.02, graph=True)
    c.run_tile_ticks(20, 0.02, graph=True)
    c.run_tile_ticks(3, 0.02, graph=False)
    c.run_tile_ticks(2, 0.02, graph=False, streams=3)
    assert np.array_equal(a.tile_hashes(), c.tile_hashes())


@pytest.mark.parametrize("rows", [1, 4, 16, 32, 64])
@pytest.mark.parametrize("order", [0, 1])
def test_every_tuning_gives_the_same_bytes(gpu, rows, order):
    tiles, sides, edges = mixed_tiles()
    ref = Batch(sides, open_edges=edges)
    load(ref, tiles)
    ref.run_ticks(19, 0.02)
    b = Batch(sides, open_edges=edges)
    b.set_tuning(rows, order)
    load(b, tiles)
    b.run_ticks(19, 0.02)
    assert np.array_equal(ref.tile_hashes(), b.tile_hashes())


def test_autotune_leaves_the_state_as_it_was(gpu):
    tiles, sides, edges = mixed_tiles()
    a = Batch(sides, open_edges=edges)
    b = Batch(sides, open_edges=edges)
    load(a, tiles)
    load(b, tiles)
    a.run_ticks(5, 0.02)
    b.run_ticks(5, 0.02)
    chosen = b.autotune(0.02, trial_ticks=3)
    assert chosen["block_rows"] in (1, 4, 16, 32, 64) and chosen["order"] in (0, 1)
    assert chosen["us_per_tick"] > 0
    a.run_ticks(9, 0.02)
    b.run_ticks(9, 0.02)
    assert np.array_equal(a.tile_hashes(), b.tile_hashes())
    # the tuning is cached per size histogram: a second batch of the same sizes reuses it
    c = Batch(sides, open_edges=edges)
    load(c, tiles)
    assert c.autotune(0.02, trial_ticks=3) == chosen


@pytest.mark.parametrize("rows", [16, 32, 64])
def test_zero_apart_gives_the_same_bytes(gpu, rows):
    """The march's zero-apart variant (the autotuner's knob) on a plain batch of the batched
    configuration's tiles (dry land, a column each: zero depths and momenta everywhere): every
    tile's bytes equal the bare intrinsics' after 120 ticks, and sampled tiles the oracle's."""
    tiles = workloads.tiles_4096(24)
    sides = [(t.nx, t.ny) for t in tiles]
    out = []
    for zg in (0, 1):
        b = Batch(sides)
        b.set_tuning(rows, 1, zero_apart=zg)
        assert b.tuning()["zero_apart"] == zg
        load(b, tiles, source=False)
        b.run_ticks(120, 0.01)
        out.append(b.tile_hashes())
        b.close()
    assert np.array_equal(out[0], out[1])
    for k in (0, 11, 23):
        r = oracle_tile(tiles[k], 0, 120, 0.01, source=False)
        assert int(out[1][k]) == r.state_hash(), f"tile {k} {sides[k]}"


def test_tiles_configuration_sample(gpu):
    # The batched configuration's tile-size distribution, 48 tiles, 200 ticks: every tile's
    # hash against the oracle.
    tiles = workloads.tiles_4096(48)
    sides = [(t.nx, t.ny) for t in tiles]
    b = Batch(sides)
    load(b, tiles, source=False)
    b.autotune(0.01)
    b.run_ticks(200, 0.01)
    hashes = b.tile_hashes()
    for k in range(0, 48, 5):
        r = oracle_tile(tiles[k], 0, 200, 0.01, source=False)
        assert int(hashes[k]) == r.state_hash(), f"tile {k} {sides[k]}"


@pytest.mark.parametrize("rows", [16, 1])
def test_one_tile_wakes_with_a_new_state(gpu, rows):
    """A tile's state written between ticks (the tile-start upload of a tile waking from the baked
    solve): that tile equals an oracle written at the same tick, and every other tile, its
    pending records and its ledger included, equals its oracle as if nothing happened."""
    tiles, sides, edges = mixed_tiles()
    b = Batch(sides, open_edges=edges)
    b.set_tuning(rows, 0)
    load(b, tiles)
    b.run_ticks(11, 0.02)
    wake = 2
    nx, ny = sides[wake]
    x, y = np.meshgrid(np.arange(nx), np.arange(ny))
    h_new = 0.5 + 0.3 * ((x + 2 * y) % 7 == 0).ravel()
    hu_new = np.full(nx * ny, 0.05)
    b.write_tile_state(wake, h_new, hu_new, np.zeros(nx * ny))
    b.run_ticks(13, 0.02)
    ledgers = b.ledgers()
    for k, t in enumerate(tiles):
        r = oracle.RefStep(oracle.Grid(t.nx, t.ny, t.cell_m, open_edges=edges[k]))
        r.set_bed(t.bed)
        r.set_source(t.source)
        r.write_state(t.h, t.hu, t.hv)
        r.run_steps(11, 0.02)
        if k == wake:
            r.write_state(h_new, hu_new, np.zeros(nx * ny))
        r.run_steps(13, 0.02)
        got, want = b.read_tile_bits(k), r.read_state_bits()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"tile {k}"
        led = r.read_ledger()
        for key in ("source_m3", "open_edge_out_m3", "roundoff_m3", "time_s", "steps"):
            assert ledgers[k][key] == led[key], (k, key)
    with pytest.raises(Exception):
        b.write_tile_state(wake, np.zeros(3))  # a state that does not fit the tile
    b.close()

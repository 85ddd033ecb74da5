"""record() on a caller's stream and into a CUDA graph; the benchmark workloads at full size.

Every per-tick quantity lives on the device, so a captured graph of tick launches replays
correctly any number of times. At the benchmark's full sizes the oracle checks the first ticks bit
for bit and the whole run is held to size-independent properties: the same bytes twice, and the
water's balance.
"""
from __future__ import annotations

import numpy as np
import pytest

import cases
from pairs import assert_same, make_pair
from game_engine_gb300 import water_live as wl, workloads

pytestmark = pytest.mark.gpu
INF = float("inf")


def test_enqueue_on_a_caller_stream(gpu):
    import torch
    s = cases.slope(False)
    dev, ref = make_pair(s)
    stream = torch.cuda.Stream()
    assert dev.record(stream.cuda_stream, 37, INF)
    stream.synchronize()
    ref.run_steps(37, INF)
    assert_same(dev, ref, "caller stream")


def test_graph_capture_replays(gpu):
    import torch
    s = cases.slope(False)
    dev, ref = make_pair(s)
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        assert dev.record(torch.cuda.current_stream().cuda_stream, 5, INF)
    # Capture records the launches without running them; each replay is five ticks, and a
    # replay of an odd count flips the copy on the device, where every launch reads it.
    for _ in range(7):
        graph.replay()
    torch.cuda.synchronize()
    ref.run_steps(35, INF)
    assert_same(dev, ref, "graph replays")


def tile_case(t):
    return dict(nx=t.nx, ny=t.ny, cell_m=t.cell_m, bed=t.bed, h=t.h, source=t.source)


def test_plain_256_thousand_ticks_hash(gpu):
    # The plain configuration: 256 x 256 fBm, a 2 m column, 1000 ticks at max_dt 0.01 s.
    t = workloads.plain_256()
    dev, ref = make_pair(tile_case(t))
    assert dev.run_steps(1000, 0.01)
    ref.run_steps(1000, 0.01)
    assert_same(dev, ref, "plain_256")


def test_plain_2048_first_ticks_bit_exact(gpu):
    t = workloads.plain_2048()
    dev, ref = make_pair(tile_case(t))
    assert dev.run_steps(3, 0.01)
    ref.run_steps(3, 0.01)
    assert_same(dev, ref, "plain_2048, 3 ticks")


@pytest.mark.parametrize("fixed", [False, True])
def test_a_tile_of_more_items_than_warps(gpu, fixed):
    """1024 x 2080 (32 x 130 items of 32 x 16 rows, more than the device holds warps, so warps take
    items in rounds, the last round part-filled): open west and south edges, rain with sinks, 40
    ticks, every state word, record and ledger byte against the oracle."""
    nx, ny = 1024, 2080
    bed = workloads.fbm(nx, ny, 8.0, 77)
    rng = np.random.default_rng(77)
    h = rng.uniform(0.0, 0.6, nx * ny)
    source = np.where(rng.random(nx * ny) < 0.05, -2e-3, 1e-3)
    c = dict(nx=nx, ny=ny, cell_m=1.0, bed=bed, h=h, source=source, open_edges=5)
    dev, ref = make_pair(c, fixed=fixed, rows=16)
    for k in (1, 39):
        assert dev.run_steps(k, 0.01), dev.error
        ref.run_steps(k, 0.01)
        assert_same(dev, ref, f"1024x2080 after +{k}")
    assert dev.read_ledger()["open_edge_out_m3"] != 0.0


def test_plain_2048_full_run_properties(gpu):
    # 500 ticks of rain: the same bytes twice, and the ledger's balance of the water.
    from pairs import config
    t = workloads.plain_2048()
    c = tile_case(t)
    hashes = []
    for _ in range(2):
        dev = wl.DeviceStep()
        assert dev.create(config(c)), dev.error
        assert dev.set_bed(c["bed"]) and dev.set_source(c["source"])
        assert dev.write_state(c["h"], np.zeros(t.cells), np.zeros(t.cells))
        h0 = dev.read_state()[0]
        assert dev.run_steps(500, 0.01)
        hashes.append(dev.state_hash())
    assert hashes[0] == hashes[1] != 0
    h = dev.read_state()[0]
    led = dev.read_ledger()
    assert led["steps"] == 500
    before = h0.sum()
    after = h.sum()
    balance = after - before - led["source_m3"] - led["roundoff_m3"]
    involved = before + abs(led["source_m3"])
    assert abs(balance) <= 500 * 2.0 ** -24 * involved
    assert led["source_m3"] > 0


def test_a_wait_past_its_limit_is_a_timeout_and_the_step_stays_usable(gpu, monkeypatch):
    # Failure detection without a fault: every wait on the device has a limit (WLCUDA_WAIT_S).
    # A wait that passes it returns WL_ERR_TIMEOUT's message, nothing hangs, and the work it
    # waited for finishes; the next call waits for it and the bytes are those of the whole run.
    t = workloads.plain_2048(1024)
    ref = wl.DeviceStep()
    assert ref.create(wl.Config(t.nx, t.ny, t.cell_m))
    ref.set_bed(t.bed), ref.set_source(t.source), ref.write_state(t.h, t.hu, t.hv)
    assert ref.run_steps(300, workloads.MAX_DT)
    want = ref.state_hash()
    dev = wl.DeviceStep()
    assert dev.create(wl.Config(t.nx, t.ny, t.cell_m))
    dev.set_bed(t.bed), dev.set_source(t.source), dev.write_state(t.h, t.hu, t.hv)
    monkeypatch.setenv("WLCUDA_WAIT_S", "0.000001")
    assert not dev.run_steps(300, workloads.MAX_DT)
    assert "wait limit" in dev.error
    monkeypatch.delenv("WLCUDA_WAIT_S")
    assert dev.state_hash() == want

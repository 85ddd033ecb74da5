"""The tick queue (the design of water_live.md:76-94, ADR-0081) against the oracle, bit for bit.

A queued tick takes the sub-steps the oracle's advance takes for the same length, with its events
written into the planes at its start, so after every tick has landed the state's four planes, the
records and the ledger's sums equal the oracle's advance-per-tick run. The same bytes come out
whatever number of slots each call runs ("the same bytes at any frame rate"), from a captured
graph of slots, and through a ring that wraps; idle slots change nothing; each landed tick's
read-back record carries the oracle's sub-step count.
"""
from __future__ import annotations

import numpy as np
import pytest

import cases
from pairs import bits, make_pair
from game_engine_gb300.tick_queue import (EVENT_BED, EVENT_MANNING, EVENT_SOURCE, EVENT_STATE,
                                          ERR_REFUSED, Event, TickQueue)

pytestmark = pytest.mark.gpu
TICK = float(np.float32(1.0 / 60.0))
LEDGER_SUMS = ("source_m3", "open_edge_out_m3", "roundoff_m3", "time_s", "steps")


def plan_for(c, n_ticks, seed):
    """(tick, length, events) for n ticks of 1/60 s: bed, source and Manning patches, a tick of
    no length that carries an event, and two overlapping patches in one tick."""
    rng = np.random.default_rng(seed)
    nx, ny = c["nx"], c["ny"]
    plan = []
    for t in range(n_ticks):
        events = []
        length = TICK
        if t % 6 == 3:
            w, h = int(rng.integers(1, min(nx, 9) + 1)), int(rng.integers(1, min(ny, 7) + 1))
            x0, y0 = int(rng.integers(0, nx - w + 1)), int(rng.integers(0, ny - h + 1))
            events.append(Event(EVENT_BED, x0, y0, rng.uniform(0.0, 0.4, (h, w))))
        if t % 6 == 5 and c.get("source") is not None:
            events.append(Event(EVENT_SOURCE, 2, 3, np.full((4, 5), 3e-3)))
        if t % 9 == 7 and c.get("manning") is not None:
            events.append(Event(EVENT_MANNING, 0, 0, np.full((ny, 3), 0.05)))
        if t % 10 == 9:
            length = 0.0
            events.append(Event(EVENT_BED, 1, 1, np.full((2, 2), 0.7)))
        if t % 10 == 4:
            events.append(Event(EVENT_BED, 0, 0, np.full((3, 3), 0.2)))
            events.append(Event(EVENT_BED, 1, 1, np.full((3, 3), 0.3)))  # the later one wins
        plan.append((1000 + t, length, events))
    return plan


def oracle_run(ref, c, plan, compensate=False):
    """The oracle: each tick's events into its planes, then advance(length). Returns the steps."""
    planes = {EVENT_BED: np.asarray(c["bed"], np.float64).astype(np.float32)}
    if c.get("source") is not None:
        planes[EVENT_SOURCE] = np.asarray(c["source"], np.float64).astype(np.float32)
    if c.get("manning") is not None:
        planes[EVENT_MANNING] = np.asarray(c["manning"], np.float64).astype(np.float32)
    nx, ny = c["nx"], c["ny"]
    steps = []
    for _, length, events in plan:
        for e in events:
            v = np.asarray(e.values, np.float32)
            if e.kind == EVENT_STATE:
                oracle_state_event(ref, nx, ny, e)
                continue
            p = planes[e.kind].reshape(ny, nx)
            p[e.y0:e.y0 + v.shape[0], e.x0:e.x0 + v.shape[1]] = v
        for kind in {e.kind for e in events} - {EVENT_STATE}:
            wide = planes[kind].astype(np.float64)  # f32 values widen exactly; datum 0
            {EVENT_BED: lambda: ref.set_bed(wide, 0.0),
             EVENT_SOURCE: lambda: ref.set_source(wide, 1, compensate),
             EVENT_MANNING: lambda: ref.set_manning(wide)}[kind]()
        steps.append(ref.advance(length)[0] if length > 0 else 0)
    return steps


def oracle_state_event(ref, nx, ny, e):
    """A state event in the oracle: the flush (dt_main with max_dt 0), the rectangle's h, hu, hv
    written and its remainder zeroed, then prime_main of the new state."""
    ref.run_length_pass(0.0)
    planes = ref.read_state_bits().reshape(4, ny, nx).copy()
    v = np.asarray(e.values, np.float32)
    h, w = v.shape[-2:]
    planes[0:3, e.y0:e.y0 + h, e.x0:e.x0 + w] = v
    planes[3, e.y0:e.y0 + h, e.x0:e.x0 + w] = 0.0
    ref.write_planes(planes.ravel())
    ref.prime()


def lake_patch(c, x0, y0, w, h, level):
    """A rectangle of a lake at rest at `level` over the case's bed: (3, h, w) values."""
    bed = np.asarray(c["bed"], np.float64).astype(np.float32).reshape(c["ny"], c["nx"])
    depth = np.maximum(np.float32(level) - bed[y0:y0 + h, x0:x0 + w], 0.0)
    return np.stack([depth, np.zeros_like(depth), np.zeros_like(depth)])


def device_run(q, n_ticks, partition, most_calls=20000):
    """Slots in calls of the partition's sizes, in turn, until n ticks have landed."""
    k = 0
    for _ in range(most_calls):
        st = q.status()
        if st["landed"] >= n_ticks:
            return
        assert q.run_slots(partition[k % len(partition)]), q.error
        k += 1
    raise AssertionError("the queue did not land its ticks")


def assert_same_after_ticks(dev, ref, what):
    a, b = dev.read_state_bits(), ref.read_state_bits()
    diff = np.nonzero(bits(a) != bits(b))[0]
    assert diff.size == 0, f"{what}: {diff.size} state words differ, first at {diff[:5]}"
    # The oracle's advance ends with a flush (the records' volumes folded into the ledger and
    # cleared); read_ledger flushes the device's, so the records compare after it.
    la, lb = dev.read_ledger(), ref.read_ledger()
    for k in LEDGER_SUMS:
        assert la[k] == lb[k], (what, k, la[k], lb[k])
    assert np.array_equal(bits(dev.read_partials_bits()), bits(ref.read_partials_bits())), what


@pytest.mark.parametrize("case", ["slope", "basin"])
@pytest.mark.parametrize("partition", [[1], [3, 1, 7, 2], [200]])
def test_queued_ticks_equal_advance_per_tick(gpu, case, partition):
    c = cases.slope(False) if case == "slope" else cases.closed_basin()
    dev, ref = make_pair(c)
    n = 24
    plan = plan_for(c, n, seed=11)
    want_steps = oracle_run(ref, c, plan)
    q = TickQueue(dev, records=32, arena_values=4096, max_events=64)
    for tick, length, events in plan:
        assert q.push(tick, length, events), q.error
    device_run(q, n, partition)
    assert_same_after_ticks(dev, ref, f"{case} {partition}")
    landed = q.landed(0, n)
    assert [r["tick"] for r in landed] == [t for t, _, _ in plan]
    assert [r["substeps"] for r in landed] == want_steps
    assert [r["events"] for r in landed] == [len(e) for _, _, e in plan]
    for r in landed:
        if r["substeps"]:
            assert 0.0 < r["shortest_s"] <= r["longest_s"] <= TICK
    st = q.status()
    assert st == dict(pushed=n, begun=n, landed=n, active=0, substeps=st["substeps"], dropped=0,
                      frozen=0, freezes=0)
    # Idle slots change nothing.
    h = dev.state_hash()
    assert q.run_slots(9), q.error
    assert dev.state_hash() == h and q.status()["landed"] == n
    q.close()


def test_the_queue_owns_the_clock(gpu):
    dev, ref = make_pair(cases.closed_basin())
    q = TickQueue(dev, records=8)
    assert not dev.run_steps(1, 0.01) and dev.last_code == 5
    assert dev.advance(0.1) == 0
    assert not dev.set_source(np.zeros(dev.cell_count()), every=2)
    q.close()
    # Without the queue, the step's own calls again, and the clock free-running (no time left).
    assert dev.run_steps(3, float("inf")), dev.error
    ref.run_steps(3, float("inf"))
    a, b = dev.read_state_bits(), ref.read_state_bits()
    assert np.array_equal(bits(a), bits(b))
    assert dev.read_ledger()["remaining_s"] == float("inf")


def test_refusals_keep_the_queue_whole(gpu):
    c = cases.slope(False)
    dev, _ = make_pair(c)
    q = TickQueue(dev, records=2, arena_values=64, max_events=4)
    big = Event(EVENT_BED, 0, 0, np.zeros((9, 9)))  # 81 values: more than the arena
    assert not q.push(1, TICK, [big]) and q.last_code == 2
    off = Event(EVENT_BED, 45, 0, np.zeros((1, 4)))  # leaves the 48-wide grid
    assert not q.push(1, TICK, [off]) and q.last_code == 2
    assert q.push(1, TICK) and q.push(2, TICK)
    assert not q.push(3, TICK) and q.last_code == ERR_REFUSED  # two records in flight
    assert q.status()["pushed"] == 2
    assert q.run_slots(1), q.error  # begins tick 1: its record's place is free
    assert q.push(3, TICK), q.error
    q.close()
    d2, _ = make_pair(cases.closed_basin())  # no source, no Manning
    q2 = TickQueue(d2, records=4)
    assert not q2.push(1, TICK, [Event(EVENT_SOURCE, 0, 0, np.zeros((1, 1)))])
    assert q2.last_code == 8
    q2.close()


def test_a_ring_that_wraps(gpu):
    c = cases.slope(False)
    dev, ref = make_pair(c)
    n = 150
    plan = plan_for(c, n, seed=5)
    want = oracle_run(ref, c, plan)
    q = TickQueue(dev, records=4, arena_values=256, max_events=8)
    k = 0
    for _ in range(100000):
        while k < n and q.push(*plan[k]):
            k += 1
        if k < n:
            assert q.last_code == ERR_REFUSED, q.error
        if q.status()["landed"] == n:
            break
        assert q.run_slots(3), q.error
    assert q.status()["landed"] == n
    assert_same_after_ticks(dev, ref, "wrapped")
    landed = q.landed(n - 4, 4)
    assert [r["substeps"] for r in landed] == want[-4:]
    assert q.landed(0, 1) is None  # landing 0 is no longer held
    q.close()


def test_slots_from_a_captured_graph(gpu):
    import torch
    c = cases.closed_basin()
    dev, ref = make_pair(c)
    n = 12
    plan = plan_for(c, n, seed=3)
    oracle_run(ref, c, plan)
    q = TickQueue(dev, records=16)
    for p in plan:
        assert q.push(*p), q.error
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        assert q.enqueue_slots(torch.cuda.current_stream().cuda_stream, 4)
    for _ in range(2000):
        graph.replay()
        torch.cuda.synchronize()
        if q.status()["landed"] == n:
            break
    assert q.status()["landed"] == n
    assert_same_after_ticks(dev, ref, "graph")
    q.close()


def test_a_new_state_is_refused_while_queued(gpu):
    dev, _ = make_pair(cases.closed_basin())
    q = TickQueue(dev, records=4)
    n = dev.cell_count()
    assert not dev.write_state(np.zeros(n), np.zeros(n), np.zeros(n)) and dev.last_code == 5
    q.close()
    assert dev.write_state(np.zeros(n), np.zeros(n), np.zeros(n)), dev.error


@pytest.mark.parametrize("rows", [16, 4, 1])
def test_a_batch_queue_equals_advance_per_tile(gpu, rows):
    """A domain of uneven tiles: each queued tick advances every tile by its length, each tile by
    its own sub-steps, with per-tile events; every tile equals its oracle's advance-per-tick run,
    and each landing counts the slots of its slowest tile."""
    from game_engine_gb300.batch import Batch, BatchError
    from test_batch_gpu import load, mixed_tiles
    import oracle
    tiles, sides, edges = mixed_tiles()
    b = Batch(sides, open_edges=edges)
    b.set_tuning(rows, 0)
    load(b, tiles)
    refs = []
    for k, t in enumerate(tiles):
        r = oracle.RefStep(oracle.Grid(t.nx, t.ny, t.cell_m, open_edges=edges[k]))
        r.set_bed(t.bed)
        r.set_source(t.source)
        r.write_state(t.h, t.hu, t.hv)
        refs.append(r)
    beds = [np.asarray(t.bed, np.float64).astype(np.float32) for t in tiles]
    srcs = [np.asarray(t.source, np.float64).astype(np.float32) for t in tiles]
    plan = []
    for tick in range(14):
        events, length = [], TICK
        if tick == 3:
            events = [Event(EVENT_BED, 2, 1, np.full((3, 4), 0.9), tile=0),
                      Event(EVENT_BED, 10, 20, np.full((5, 5), 0.1), tile=2)]
        if tick == 5:
            events = [Event(EVENT_SOURCE, 0, 0, np.full((4, 4), 5e-3), tile=1)]
        if tick == 7:
            length = 0.0
            events = [Event(EVENT_BED, 0, 0, np.full((2, 3), 0.5), tile=4)]
        plan.append((tick, length, events))
    want = []
    for tick, length, events in plan:
        for e in events:
            v = np.asarray(e.values, np.float32)
            nx, ny = sides[e.tile]
            p = (beds if e.kind == EVENT_BED else srcs)[e.tile].reshape(ny, nx)
            p[e.y0:e.y0 + v.shape[0], e.x0:e.x0 + v.shape[1]] = v
            if e.kind == EVENT_BED:
                refs[e.tile].set_bed(beds[e.tile].astype(np.float64))
            else:
                refs[e.tile].set_source(srcs[e.tile].astype(np.float64))
        want.append(max(r.advance(length)[0] for r in refs) if length > 0 else 0)
    q = TickQueue(b, records=16)
    for p in plan:
        assert q.push(*p), q.error
    with pytest.raises(BatchError):
        b.run_ticks(1, 0.01)  # the queue owns the clocks
    device_run(q, len(plan), [2, 5, 1])
    ledgers = b.ledgers()
    for k, r in enumerate(refs):
        got, exp = b.read_tile_bits(k), r.read_state_bits()
        assert np.array_equal(got.view(np.uint32), exp.view(np.uint32)), f"tile {k} {sides[k]}"
        led = r.read_ledger()
        for key in LEDGER_SUMS:
            assert ledgers[k][key] == led[key], (k, key)
    assert [x["substeps"] for x in q.landed(0, len(plan))] == want
    q.close()
    b.run_ticks(1, 0.01)  # the batch's own ticks again
    b.close()


@pytest.mark.parametrize("form", ["fixed", "stored_faces", "compensate"])
def test_queued_ticks_in_the_other_forms(gpu, form):
    """The fixed arithmetic, the stored-faces form and the compensated source through the queue,
    a waking state among the events: the same bytes as the oracle's advance per tick."""
    c = cases.slope(False)
    kw = {"fixed": dict(fixed=True), "stored_faces": dict(stored_faces=True),
          "compensate": dict(compensate=True)}[form]
    dev, ref = make_pair(c, **kw)
    n = 10
    plan = plan_for(c, n, seed=23)
    if form == "compensate":
        # a source event resets nothing of the remainder: the oracle's set_source would, so the
        # plan carries bed events alone
        plan = [(t, l, [e for e in ev if e.kind == EVENT_BED]) for t, l, ev in plan]
    # a waking state at tick 6 in every form (in the compensated one its remainder is zeroed)
    t6, l6, e6 = plan[6]
    plan[6] = (t6, l6, e6 + [Event(EVENT_STATE, 4, 3, lake_patch(c, 4, 3, 15, 9, 0.4))])
    oracle_run_kw = dict(compensate=True) if form == "compensate" else {}
    want = oracle_run(ref, c, plan, **oracle_run_kw)
    q = TickQueue(dev, records=16)
    for p in plan:
        assert q.push(*p), q.error
    device_run(q, n, [2, 3])
    assert_same_after_ticks(dev, ref, form)
    assert [r["substeps"] for r in q.landed(0, n)] == want
    q.close()


@pytest.mark.parametrize("case", ["slope", "basin"])
@pytest.mark.parametrize("partition", [[1], [3, 1, 7, 2]])
def test_a_state_event_wakes_the_tile_at_its_tick(gpu, case, partition):
    """The apply pass's waking state (water_live.md:80, ADR-0080 decision 4): lakes at rest written
    over rectangles at two ticks' boundaries, among the plan's other events, one of them in a tick
    of no length; the bytes equal the oracle's flush, write and prime between its advances."""
    c = cases.slope(False) if case == "slope" else cases.closed_basin()
    dev, ref = make_pair(c)
    n = 16
    plan = plan_for(c, n, seed=29)
    t, length, events = plan[4]
    plan[4] = (t, length, events + [Event(EVENT_STATE, 3, 2, lake_patch(c, 3, 2, 20, 11, 0.45))])
    t, length, events = plan[9]  # a tick of no length
    plan[9] = (t, length, [Event(EVENT_STATE, 0, 0, lake_patch(c, 0, 0, c["nx"], 5, 0.3))] + events)
    want = oracle_run(ref, c, plan)
    q = TickQueue(dev, records=32, arena_values=1 << 14, max_events=64)
    for p in plan:
        assert q.push(*p), q.error
    device_run(q, n, partition)
    assert_same_after_ticks(dev, ref, f"{case} state events")
    assert [r["substeps"] for r in q.landed(0, n)] == want
    q.close()


def test_a_batch_tile_wakes_from_its_baked_answer(gpu):
    """A domain of uneven tiles; at tick 3 tile 2 is woken with the baked answer (a lake at rest
    over its whole bed) by a state event while the others step on: every tile equals its oracle."""
    from game_engine_gb300.batch import Batch
    from test_batch_gpu import load, mixed_tiles
    import oracle
    tiles, sides, edges = mixed_tiles()
    b = Batch(sides, open_edges=edges)
    load(b, tiles)
    refs = []
    for k, t in enumerate(tiles):
        r = oracle.RefStep(oracle.Grid(t.nx, t.ny, t.cell_m, open_edges=edges[k]))
        r.set_bed(t.bed)
        r.set_source(t.source)
        r.write_state(t.h, t.hu, t.hv)
        refs.append(r)
    k2 = 2
    t2 = tiles[k2]
    c2 = dict(nx=t2.nx, ny=t2.ny, bed=t2.bed)
    wake = Event(EVENT_STATE, 0, 0, lake_patch(c2, 0, 0, t2.nx, t2.ny, 2.2), tile=k2)
    plan = [(tick, TICK, [wake] if tick == 3 else []) for tick in range(9)]
    for tick, length, events in plan:
        for e in events:
            oracle_state_event(refs[e.tile], *sides[e.tile], e)
        for r in refs:
            r.advance(length)
    q = TickQueue(b, records=16, arena_values=1 << 16)
    for p in plan:
        assert q.push(*p), q.error
    device_run(q, len(plan), [2, 1])
    ledgers = b.ledgers()
    for k, r in enumerate(refs):
        got, exp = b.read_tile_bits(k), r.read_state_bits()
        assert np.array_equal(got.view(np.uint32), exp.view(np.uint32)), f"tile {k} {sides[k]}"
        led = r.read_ledger()
        for key in LEDGER_SUMS:
            assert ledgers[k][key] == led[key], (k, key)
    q.close()
    b.close()


def test_a_lagging_domain_freezes_drops_and_thaws(gpu):
    """The lag control (water_live.md:90-92): with a lag limit of 4 ticks, three ticks step as
    ever; eight pushed at once put the lag past the limit, so the domain freezes as it stands and
    drops all eight, one a slot, applying their events in order (two overlapping bed patches and
    a waking state among them) and counting them; the landing that drains the queue thaws it, and
    the next two ticks step again. The bytes equal the oracle's run of the same ticks with the
    dropped ones' events applied and no advance."""
    c = cases.slope(False)
    dev, ref = make_pair(c)
    q = TickQueue(dev, records=16, arena_values=1 << 14, max_events=64)
    assert q.set_limits(4, 0), q.error
    first = [(t, TICK, []) for t in range(3)]
    burst = [(10 + t, TICK, []) for t in range(8)]
    burst[1] = (11, TICK, [Event(EVENT_BED, 2, 2, np.full((3, 3), 0.15))])
    burst[4] = (14, TICK, [Event(EVENT_BED, 3, 3, np.full((3, 3), 0.25)),
                           Event(EVENT_STATE, 5, 1, lake_patch(c, 5, 1, 12, 8, 0.5))])
    last = [(30 + t, TICK, []) for t in range(2)]
    want_first = oracle_run(ref, c, first)
    for p in first:
        assert q.push(*p), q.error
    device_run(q, 3, [2])
    st = q.status()
    assert (st["dropped"], st["frozen"], st["freezes"]) == (0, 0, 0)
    oracle_run(ref, c, [(t, 0.0, e) for t, _, e in burst])  # the dropped ticks: events alone
    for p in burst:
        assert q.push(*p), q.error
    device_run(q, 11, [3, 1])
    st = q.status()
    assert (st["dropped"], st["frozen"], st["freezes"]) == (8, 0, 1)
    rec = q.landed(3, 8)
    assert [r["dropped"] for r in rec] == [1] * 8
    assert [r["substeps"] for r in rec] == [0] * 8
    assert [r["dropped_total"] for r in rec] == list(range(1, 9))
    assert rec[0]["lag"] == 8 and [r["frozen"] for r in rec] == [1] * 7 + [0]
    assert [r["events"] for r in rec] == [len(e) for _, _, e in burst]
    want_last = oracle_run(ref, c, last)
    for p in last:
        assert q.push(*p), q.error
    device_run(q, 13, [1])
    rec = q.landed(11, 2)
    assert [r["dropped"] for r in rec] == [0, 0]
    assert [r["substeps"] for r in rec] == want_last
    assert [r["substeps"] for r in q.landed(0, 3)] == want_first
    assert_same_after_ticks(dev, ref, "frozen and thawed")
    # A second burst freezes the domain again; the drops add up across freezes.
    again = [(40 + t, TICK, [Event(EVENT_BED, t, 0, np.full((1, 2), 0.05 * t))]) for t in range(6)]
    oracle_run(ref, c, [(t, 0.0, e) for t, _, e in again])
    for p in again:
        assert q.push(*p), q.error
    device_run(q, 19, [4])
    st = q.status()
    assert (st["dropped"], st["frozen"], st["freezes"]) == (14, 0, 2)
    assert [r["dropped_total"] for r in q.landed(13, 6)] == list(range(9, 15))
    assert_same_after_ticks(dev, ref, "frozen twice")
    q.close()


def test_max_slots_caps_a_call(gpu):
    dev, _ = make_pair(cases.closed_basin())
    q = TickQueue(dev, records=16)
    assert q.set_limits(0, 3), q.error
    for t in range(10):
        assert q.push(t, TICK), q.error
    before = int(dev.read_ledger_bits()[10])
    assert q.run_slots(100), q.error
    taken = int(dev.read_ledger_bits()[10]) - before
    assert taken == 3  # three slots, each a sub-step of a tick in flight
    assert q.set_limits(0, 0), q.error
    assert q.run_slots(5), q.error
    assert int(dev.read_ledger_bits()[10]) - before == 8
    q.close()

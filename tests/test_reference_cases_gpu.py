"""The reference's device cases (systems/water_live/tests/water_live_device_tests.cpp), run on the
CUDA path and held to the FP64 reference CPU tick (the oracle's Solver64, byte-equal to the
reference's own build) with the reference's stated bounds: about one float ulp of the water
involved a step, S x 2^-23 after S steps (device_tests.cpp:1-9).
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import cases
import oracle
from pairs import block_rows, config
from game_engine_gb300 import water_live as wl

pytestmark = pytest.mark.gpu
ULP = 2.0 ** -24
RATIO = 2.0 ** 29
INF = float("inf")


def device(c, fixed=False, datum=0.0, raise_m=0.0, stored_faces=False):
    s = wl.DeviceStep()
    assert s.create(config(c), wl.StepOptions(ops=wl.OPS_FIXED if fixed else wl.OPS_NATIVE,
                                              stored_faces=stored_faces)), s.error
    n = c["nx"] * c["ny"]
    assert s.set_bed(c["bed"] + raise_m, datum)
    if c.get("manning") is not None:
        assert s.set_manning(c["manning"])
    if c.get("source") is not None:
        assert s.set_source(c["source"])
    assert s.write_state(c["h"], np.zeros(n), np.zeros(n)), s.error
    return s


def reference(c):
    g = oracle.Grid(c["nx"], c["ny"], c["cell_m"], open_edges=c.get("open_edges", 0))
    r = oracle.Solver64(g)
    r.set_state(c["h"])
    r.set_inputs(c["bed"], c.get("manning"), c.get("source"))
    return r


def lake_run(c, fixed, raise_m, datum):
    s = device(c, fixed, datum, raise_m)
    h0, _, _ = s.read_state()
    steps = s.advance(20.0)
    assert steps > 0, s.error
    h, hu, hv = s.read_state()
    z = (c["bed"] + raise_m - datum).astype(np.float32).astype(np.float64)
    wet = h > 0
    drift = np.max(np.abs(h + z - (z + h0.astype(np.float32).astype(np.float64)))[wet])
    u = np.where(wet, hu / np.where(wet, h, 1), 0)
    v = np.where(wet, hv / np.where(wet, h, 1), 0)
    moved = int(np.sum((h != h0) | (hu != 0) | (hv != 0)))
    return dict(steps=steps, moved=moved, drift=drift, fastest=np.max(np.hypot(u, v)),
                roundoff=s.read_ledger()["roundoff_m3"], hash=s.state_hash())


@pytest.mark.parametrize("fixed", [False, True])
def test_exact_lake_stays_exactly_at_rest_at_any_datum(gpu, fixed):
    lake = cases.exact_lake()
    low = lake_run(lake, fixed, 0.0, 0.0)
    high = lake_run(lake, fixed, 2000.0, 2000.0)
    assert low["steps"] > 500
    assert low["moved"] == 0 and high["moved"] == 0
    assert low["roundoff"] == 0.0
    assert low["hash"] == high["hash"]


@pytest.mark.parametrize("fixed", [False, True])
def test_inexact_lake_at_rest_to_single_precision(gpu, fixed):
    lake = cases.inexact_lake()
    low = lake_run(lake, fixed, 0.0, 0.0)
    high = lake_run(lake, fixed, 2000.0, 2000.0)
    world = lake_run(lake, fixed, 2000.0, 0.0)
    assert low["drift"] <= 1e-13 * RATIO
    assert low["fastest"] <= 1e-11 * RATIO
    assert low["hash"] == high["hash"]
    assert world["moved"] > 0
    assert world["drift"] >= 0.5 / 8192.0


def dam_run(nx, hr, fixed):
    c = cases.dam(nx, hr)
    ref = reference(c)
    ref.advance(6.0)
    s = device(c, fixed)
    steps = s.advance(6.0)
    h, _, _ = s.read_state()
    rh, _, _ = ref.state()
    xs = (np.arange(nx) + 0.5) * c["cell_m"]
    exact = np.array([dam_depth(x, 6.0, 0.005, hr) for x in xs])
    before = np.sum(c["h"].astype(np.float32).astype(np.float64))
    return dict(steps=steps, l1=np.sum(np.abs(h - exact)) / np.sum(exact),
                l1_ref=np.sum(np.abs(h - rh)) / np.sum(rh), linf_ref=np.max(np.abs(h - rh)),
                min=h.min(), volume=abs(np.sum(h) - before) / before)


def stoker_cm(hl, hr, g=9.81):  # device_tests.cpp:65-84 (SWASHES 4.1.1)
    sl = math.sqrt(g * hl)

    def f(c):
        a = sl - c
        b = c * c - g * hr
        return -8.0 * g * hr * c * c * a * a + b * b * (c * c + g * hr)

    lo, hi = math.sqrt(g * hr), sl
    flo = f(lo)
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if (f(mid) > 0.0) == (flo > 0.0):
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def dam_depth(x, t, hl, hr, x0=5.0, g=9.81):  # device_tests.cpp:86-101
    sl = math.sqrt(g * hl)
    if x <= x0 - t * sl:
        return hl
    fan = 4.0 / (9.0 * g) * (sl - (x - x0) / (2.0 * t)) ** 2
    if hr == 0.0:
        return fan if x <= x0 + 2.0 * t * sl else 0.0
    cm = stoker_cm(hl, hr)
    xb = x0 + t * (2.0 * sl - 3.0 * cm)
    xc = x0 + t * 2.0 * cm * cm * (sl - cm) / (cm * cm - g * hr)
    if x <= xb:
        return fan
    if x <= xc:
        return cm * cm / g
    return hr


@pytest.mark.parametrize("hr,finest", [(0.001, 0.0045), (0.0, 0.0058)], ids=["stoker", "ritter"])
@pytest.mark.parametrize("fixed", [False, True])
def test_dam_breaks_as_the_reference(gpu, hr, finest, fixed):
    r = [dam_run(nx, hr, fixed) for nx in (200, 400, 800)]
    assert math.log2(r[0]["l1"] / r[1]["l1"]) >= 0.5
    assert math.log2(r[1]["l1"] / r[2]["l1"]) >= 0.5
    assert r[2]["l1"] <= finest
    assert r[2]["min"] >= 0.0
    deep_ulp = 2.0 ** -31
    for x in r:
        assert x["linf_ref"] <= 8.0 * math.sqrt(x["steps"]) * deep_ulp
        assert x["l1_ref"] <= x["steps"] * 2.0 * ULP
        assert x["volume"] <= x["steps"] * ULP


@pytest.mark.parametrize("all_open", [False, True])
@pytest.mark.parametrize("fixed", [False, True])
def test_water_is_counted_as_the_reference_counts_it(gpu, all_open, fixed):
    c = cases.slope(all_open)
    ref = reference(c)
    for _ in range(6):
        ref.advance(10.0)
    ref_volume = ref.volume()
    ref_out = ref.ledger()["open_edge_out_m3"]
    s = device(c, fixed)
    h, _, _ = s.read_state()
    initial = np.sum(h) * 0.25
    was_wet = h > 0
    steps = 0
    lowest = 0.0
    for _ in range(6):
        steps += s.advance(10.0)
        h, hu, hv = s.read_state()
        lowest = min(lowest, h.min())
    volume = np.sum(h) * 0.25
    led = s.read_ledger()
    balance = volume + led["open_edge_out_m3"] - initial - led["source_m3"] - led["roundoff_m3"]
    involved = initial + abs(led["source_m3"])
    assert lowest >= 0.0
    assert int(np.sum(~was_wet & (h > 0))) > 200
    drained = sum(h[y * 48 + x] == 0.0 for y in range(28, 32) for x in range(30, 34))
    assert drained > 0
    assert led["open_edge_out_m3"] > 0.0 if not all_open else True
    assert abs(balance) <= steps * ULP * involved
    assert led["roundoff_m3"] <= 1e-15 * RATIO * initial
    # The reference's Manning uses its own cube root; the bounds are the reference's.
    assert abs(volume - ref_volume) <= steps * 2.0 * ULP * involved
    assert abs(led["open_edge_out_m3"] - ref_out) <= steps * 2.0 * ULP * involved
    rh, rhu, _ = ref.state()
    assert np.sum(np.abs(h - rh)) / np.sum(np.abs(rh)) <= steps * 2.0 * ULP
    assert np.sum(np.abs(hu - rhu)) / np.sum(np.abs(rhu)) <= steps * 2.0 * ULP


@pytest.mark.parametrize("fixed", [False, True])
def test_same_bytes_twice_and_stored_faces(gpu, fixed):
    # The stored-faces form (every face stored once, then gathered: the block shape) against the
    # march, twice.
    c = cases.slope(False)
    hashes = []
    for stored, rows in ((False, 16), (False, 16), (True, None)):
        with block_rows(rows):
            s = device(c, fixed, stored_faces=stored)
        assert s.run_steps(400, INF)
        hashes.append(s.state_hash())
    assert hashes[0] != 0
    assert hashes[0] == hashes[1] == hashes[2]


def test_ladder_equals_one_batch(gpu):
    # device_tests.cpp:689-741: the same 400 steps read at rungs, and in one batch.
    c = cases.slope(False)
    lad = device(c)
    done = 0
    seen = []
    for rung in (1, 2, 3, 4, 8, 16, 32, 64, 128, 256, 400):
        assert lad.run_steps(rung - done, INF)
        done = rung
        seen.append((lad.state_hash(), lad.read_partials_bits().tobytes(),
                     lad.read_ledger_bits().tobytes()))
    one = device(c)
    assert one.run_steps(400, INF)
    assert one.state_hash() == seen[-1][0]


def test_closed_basin_keeps_its_water(gpu):
    c = cases.closed_basin()
    s = device(c)
    h, _, _ = s.read_state()
    before = h.sum()
    assert s.run_steps(1000, INF)
    h, hu, _ = s.read_state()
    area = 0.25 * 0.25
    bound = 1000.0 * c["nx"] * c["ny"] * ULP * 0.8 * area
    assert np.max(np.abs(hu)) > 0.01
    assert abs(h.sum() - before) * area <= bound


def test_compensated_sink_under_the_last_bit(gpu):
    # device_tests.cpp:743-787: 36,000 steps at 1/60 s; the compensated form loses what it owes
    # to two ulps of the depth.
    n = 32 * 32
    c = dict(nx=32, ny=32, cell_m=0.5, bed=np.zeros(n), h=np.ones(n))
    s = wl.DeviceStep()
    assert s.create(config(c))
    assert s.set_bed(c["bed"])
    assert s.set_source(np.full(n, -3.7e-6), 1, True)
    assert s.write_state(c["h"], np.zeros(n), np.zeros(n))
    frame = np.float32(1.0 / 60.0)
    for _ in range(36):
        assert s.run_steps(1000, float(frame))
    h, _, _ = s.read_state()
    want = 3.7e-6 * float(frame) * 36000
    assert abs((1.0 - h[n // 2]) - want) <= 2.0 * ULP

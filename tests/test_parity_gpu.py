"""The CUDA tick against the oracle, bit for bit: the state's four planes, the workgroups' records
and the ledger's bytes, on the reference's cases, both forms of the arithmetic, every block shape,
odd sizes, open edges, Manning's friction, sources (plain, coarser clock, compensated), advances
that land, zero-length steps, and the diagnosis calls.
"""
from __future__ import annotations

import numpy as np
import pytest

import cases
from pairs import assert_same, make_pair

pytestmark = pytest.mark.gpu
INF = float("inf")


def run_both(dev, ref, steps=None, advance=None, max_dt=INF):
    if advance is not None:
        a = dev.advance(advance)
        b, _ = ref.advance(advance)
        assert a == b, (a, b, dev.error)
        return a
    assert dev.run_steps(steps, max_dt), dev.error
    ref.run_steps(steps, max_dt)
    return steps


@pytest.mark.parametrize("rows", [1, 4, 16, 32, 64])
@pytest.mark.parametrize("fixed", [False, True])
def test_count_of_water_bit_exact(gpu, rows, fixed):
    s = cases.slope(False)
    dev, ref = make_pair(s, fixed=fixed, rows=rows)
    for k in (1, 1, 2, 4, 8, 48, 336):
        run_both(dev, ref, steps=k)
        assert_same(dev, ref, f"slope after +{k}")


@pytest.mark.parametrize("fixed", [False, True])
def test_exact_lake_lands_and_keeps_its_hash(gpu, fixed):
    dev, ref = make_pair(cases.exact_lake(), fixed=fixed)
    assert run_both(dev, ref, advance=20.0) == 557
    assert_same(dev, ref, "exact lake")
    assert dev.state_hash() == 6248193821885885893


@pytest.mark.parametrize("all_open", [False, True])
def test_open_edges_and_their_ledger(gpu, all_open):
    s = cases.slope(all_open)
    dev, ref = make_pair(s)
    run_both(dev, ref, advance=10.0)
    assert_same(dev, ref, "slope open edges")
    a, b = dev.read_ledger(), ref.read_ledger()
    assert a == b


@pytest.mark.parametrize("case", ["stoker", "ritter", "basin", "inexact"])
def test_reference_cases_bit_exact(gpu, case):
    c = {"stoker": cases.dam(800, 0.001), "ritter": cases.dam(400, 0.0),
         "basin": cases.closed_basin(), "inexact": cases.inexact_lake()}[case]
    dev, ref = make_pair(c)
    if case == "basin":
        run_both(dev, ref, steps=300)
    else:
        run_both(dev, ref, advance=6.0)
    assert_same(dev, ref, case)


@pytest.mark.parametrize("nx,ny", [(1, 1), (1, 37), (45, 3), (17, 17), (33, 65), (100, 70),
                                   (31, 129)])
@pytest.mark.parametrize("rows", [1, 4, 16, 32, 64])
def test_odd_sizes_and_partial_blocks(gpu, nx, ny, rows):
    x, y = cases.grid_xy(nx, ny)
    bed = (cases.mix(x, y) % 100).astype(float) / 100.0
    h = np.maximum(1.2 - bed, 0) + (cases.mix(y, x) % 7 == 0) * 0.5
    c = dict(nx=nx, ny=ny, cell_m=1.0, bed=bed, h=h, open_edges=5)
    dev, ref = make_pair(c, rows=rows)
    run_both(dev, ref, steps=60)
    assert_same(dev, ref, f"{nx}x{ny}")


@pytest.mark.parametrize("edges", [0, 9])
def test_block_shape_on_a_tile_of_more_blocks_than_sms(gpu, edges):
    """The three-phase block shape in its 256-thread CTA (a 700 x 300 tile is 22 x 19 = 418 blocks,
    more than the device has SMs; smaller launches take the 512-thread CTA, which the odd sizes
    above cover): rain with sinks, 40 ticks against the oracle."""
    nx, ny = 700, 300
    x, y = cases.grid_xy(nx, ny)
    bed = (cases.mix(x, y) % 1000).astype(float) / 400.0
    h = np.maximum(2.0 - bed, 0.0) + (cases.mix(y, x) % 5 == 0) * 0.3
    source = np.where(cases.mix(x + np.uint64(7), y) % 13 == 0, -2e-3, 5e-4)
    c = dict(nx=nx, ny=ny, cell_m=1.0, bed=bed, h=h, source=source, open_edges=edges)
    dev, ref = make_pair(c, rows=1)
    run_both(dev, ref, steps=40)
    assert_same(dev, ref, f"700x300 edges {edges}")


@pytest.mark.parametrize("every,compensate", [(1, False), (8, False), (64, False), (1, True)])
def test_slow_sink_forms(gpu, every, compensate):
    # device_tests.cpp:743-787 in small: a pond losing 3.7e-6 m/s at 1/60 s steps.
    n = 32 * 32
    c = dict(nx=32, ny=32, cell_m=0.5, bed=np.zeros(n), h=np.ones(n),
             source=np.full(n, -3.7e-6))
    dev, ref = make_pair(c, every=every, compensate=compensate)
    run_both(dev, ref, steps=777, max_dt=1.0 / 60.0)
    assert_same(dev, ref, f"sink every {every} compensate {compensate}")
    if every > 1:
        assert dev.advance(1.0) == 0  # a coarser clock is refused (water_live.cpp:600-606)


def test_compensated_spring_and_drain(gpu):
    s = cases.slope(False)
    dev, ref = make_pair(s, compensate=True)
    run_both(dev, ref, steps=300)
    assert_same(dev, ref, "compensated slope")


def test_zero_length_steps_copy_the_state(gpu):
    # An advance's batch pads with steps of no length (slang:576-585); max_dt 0 is a flush.
    s = cases.slope(False)
    dev, ref = make_pair(s)
    run_both(dev, ref, advance=0.37)
    run_both(dev, ref, steps=5, max_dt=0.0)
    assert_same(dev, ref, "zero-length")


def test_length_pass_and_diagnosis_reads(gpu):
    s = cases.slope(False)
    dev, ref = make_pair(s)
    run_both(dev, ref, steps=3)
    assert_same(dev, ref, "before the length pass")
    assert dev.run_length_pass(INF)
    ref.run_length_pass(INF)
    assert np.array_equal(dev.read_ledger_bits(), ref.read_ledger_bits())
    run_both(dev, ref, steps=2)
    assert_same(dev, ref, "after the length pass")


def test_write_state_mid_run_resets_the_ledger_and_clock(gpu):
    s = cases.slope(False)
    dev, ref = make_pair(s, every=3)
    run_both(dev, ref, steps=7)
    n = s["nx"] * s["ny"]
    rng = np.random.default_rng(3)
    h = np.maximum(rng.uniform(-0.1, 0.4, n), 0.0)
    hu = rng.uniform(-0.05, 0.05, n)
    hv = rng.uniform(-0.05, 0.05, n)
    assert dev.write_state(h, hu, hv)
    ref.write_state(h, hu, hv)
    run_both(dev, ref, steps=11)
    assert_same(dev, ref, "after a second write_state")


def test_manning_toggles(gpu):
    s = cases.slope(False)
    dev, ref = make_pair(s)
    run_both(dev, ref, steps=20)
    assert dev.set_manning(None)
    ref.set_manning(None)
    run_both(dev, ref, steps=20)
    assert dev.set_manning(s["manning"] * 2.0)
    ref.set_manning(s["manning"] * 2.0)
    run_both(dev, ref, steps=20)
    assert_same(dev, ref, "manning toggled")


def test_bed_at_a_datum(gpu):
    # set_bed takes bed - datum in double, rounded once (water_live.cpp:439-447).
    lake = cases.inexact_lake()
    c = dict(lake, bed=lake["bed"] + 2000.0)
    dev, ref = make_pair(c, datum=2000.0)
    run_both(dev, ref, advance=5.0)
    assert_same(dev, ref, "datum 2000")

"""The resident tick: a small tile (no more 32 x 16 blocks than the device holds resident CTAs)
steps a call's ticks in one cooperative launch, a grid barrier between ticks in place of the launch
boundary. Held here to the same tile stepped a launch a tick (one tick a call) bit for bit: the
state's four planes, the records and the ledger, with every flag, both forms of the arithmetic,
advance and a captured graph; and the barrier's bounded wait. (The parity suite's multi-tick runs
on small tiles go through the resident tick too, against the oracle.)"""
from __future__ import annotations

import numpy as np
import pytest

import cases
from pairs import bits, make_pair

pytestmark = pytest.mark.gpu


def same_bits(a, b, what):
    for name, x, y in (("state", a.read_state_bits(), b.read_state_bits()),
                       ("records", a.read_partials_bits(), b.read_partials_bits())):
        diff = np.nonzero(bits(x) != bits(y))[0]
        assert diff.size == 0, f"{what}: {diff.size} {name} words differ, first at {diff[:5]}"
    assert np.array_equal(a.read_ledger_bits(), b.read_ledger_bits()), f"{what}: ledger differs"


def lake_256():
    from game_engine_gb300 import workloads
    t = workloads.plain_256()
    return dict(nx=t.nx, ny=t.ny, cell_m=t.cell_m, bed=t.bed, h=t.h, source=t.source)


CASES = {
    "slope": lambda: cases.slope(),
    "slope_all_open": lambda: cases.slope(all_open=True),
    "closed_basin": cases.closed_basin,
    "exact_lake": cases.exact_lake,
    "lake_256": lake_256,
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("fixed", [False, True])
def test_resident_equals_a_launch_a_tick(gpu, name, fixed):
    c = CASES[name]()
    a, _ = make_pair(c, fixed=fixed)
    b, _ = make_pair(c, fixed=fixed)
    ticks, max_dt = 57, 0.02
    na, nb = a.tick_launches(), b.tick_launches()
    assert a.run_steps(ticks, max_dt), a.error
    for _ in range(ticks):
        assert b.run_steps(1, max_dt), b.error
    assert a.tick_launches() == na + 1  # one launch for the call's ticks
    assert b.tick_launches() == nb + ticks
    same_bits(a, b, name)
    a.destroy()
    b.destroy()


@pytest.mark.parametrize("every,compensate", [(1, True), (3, False), (4, True)])
def test_resident_source_clocks(gpu, every, compensate):
    c = cases.slope()
    a, _ = make_pair(c, every=every, compensate=compensate)
    b, _ = make_pair(c, every=every, compensate=compensate)
    assert a.run_steps(23, 0.05), a.error
    for _ in range(23):
        assert b.run_steps(1, 0.05), b.error
    same_bits(a, b, f"every {every}, compensate {compensate}")


def test_resident_advance_against_the_oracle(gpu):
    """advance's batches of ticks (resident launches) land where the oracle's advance does."""
    from pairs import assert_same
    c = cases.closed_basin()
    a, ref = make_pair(c)
    n0 = a.tick_launches()
    steps = a.advance(0.75)
    want, _ = ref.advance(0.75)
    assert steps == want and steps > 0, (steps, want, a.error)
    assert a.tick_launches() - n0 < steps  # batches of ticks, not a launch a tick
    assert_same(a, ref, "advance")


def test_resident_in_a_captured_graph(gpu):
    """A one-tile batch records its ticks into a CUDA graph: the resident launch as a graph node,
    replayed, equals the per-tick launches."""
    from game_engine_gb300.batch import Batch
    c = cases.closed_basin()
    sides = [(c["nx"], c["ny"])]
    b1 = Batch(sides, cell_m=c["cell_m"])
    b1.set_tuning(1, 0)  # the three-phase block shape, which a small tile steps resident
    b1.set_bed(np.asarray(c["bed"], np.float64))
    b1.write_state(np.asarray(c["h"], np.float64))
    b1.run_ticks(40, 0.01, graph=True)
    b1.run_ticks(40, 0.01, graph=True)
    b2 = Batch(sides, cell_m=c["cell_m"])
    b2.set_tuning(1, 0)
    b2.set_bed(np.asarray(c["bed"], np.float64))
    b2.write_state(np.asarray(c["h"], np.float64))
    for _ in range(80):
        b2.run_ticks(1, 0.01)
    assert np.array_equal(bits(b1.read_tile_bits(0)), bits(b2.read_tile_bits(0)))
    b1.close()
    b2.close()


def test_a_tile_past_the_resident_size_takes_a_launch_a_tick(gpu):
    nx = ny = 512  # 512 blocks of 32 x 16: more than the device holds resident at once
    c = dict(nx=nx, ny=ny, cell_m=1.0, bed=np.zeros(nx * ny), h=np.full(nx * ny, 0.5))
    a, _ = make_pair(c)
    n0 = a.tick_launches()
    assert a.run_steps(5, 0.01), a.error
    assert a.tick_launches() == n0 + 5


def test_the_barriers_wait_gives_up(gpu):
    """Four CTAs meet at the barrier but the last never arrives: the others' wait runs out after
    about a second, marks the error word and leaves; the context stays usable."""
    import ctypes as C
    buf = C.create_string_buffer(256)
    assert gpu.wl_resident_barrier_check(0, 4, buf, len(buf)) == 0, buf.value.decode()
    c = cases.exact_lake()
    a, _ = make_pair(c)
    assert a.run_steps(3, 0.02), a.error

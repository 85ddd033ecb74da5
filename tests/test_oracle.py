"""The oracle pinned to the reference: its published known answers and golden vectors made by the
reference's own solver (tests/golden/). CPU only.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


PINS = load("reference_pins.json")
FP64 = load("reference_fp64.json")


def refstep(oracle_mod, c, fixed=False, precision64=False):
    g = oracle_mod.Grid(c["nx"], c["ny"], c["cell_m"], open_edges=c.get("open_edges", 0))
    s = oracle_mod.RefStep(g, fixed_ops=fixed, precision64=precision64)
    z = np.zeros(g.cells)
    s.set_bed(c["bed"])
    if c.get("manning") is not None:
        s.set_manning(c["manning"])
    if c.get("source") is not None:
        s.set_source(c["source"])
    s.write_state(c["h"], z, z)
    return s


def test_fnv_empty_and_bit_sensitive(oracle_mod):
    # water_live_tests.cpp:49-55
    assert oracle_mod.hash_floats(np.zeros(0, np.float32)) == int(PINS["fnv_empty"]["hash"])
    a = np.array([1.0, 2.0], np.float32)
    b = np.array([1.0, np.nextafter(np.float32(2.0), np.float32(3.0))], np.float32)
    assert oracle_mod.hash_floats(a) != oracle_mod.hash_floats(b)


def test_stoker_800_cross_toolchain_pin(oracle_mod):
    # water_state_tests.cpp:776-789: the reference's FP64 bytes after Stoker's dam break.
    c = cases.dam(800, 0.001)
    s = oracle_mod.Solver64(oracle_mod.Grid(c["nx"], c["ny"], c["cell_m"]))
    s.set_state(c["h"])
    s.set_inputs(c["bed"])
    assert s.advance(6.0) == PINS["stoker_800_fp64"]["steps"]
    assert s.state_hash() == int(PINS["stoker_800_fp64"]["hash"])


@pytest.mark.parametrize("fixed", [False, True])
def test_exact_lake_known_answer(oracle_mod, fixed):
    # water_live.md:40-41: 557 steps and the same hash on both cards and in both op forms.
    s = refstep(oracle_mod, cases.exact_lake(), fixed=fixed)
    steps, refused = s.advance(20.0)
    assert not refused
    assert steps == PINS["exact_lake_fp32"]["steps"]
    assert s.state_hash() == int(PINS["exact_lake_fp32"]["hash"])


@pytest.mark.parametrize("fixed", [False, True])
def test_count_of_water_matches_the_card(oracle_mod, fixed):
    # water-step-on-the-card.md: 824 steps, 7.44407 m3 left, 27.9762 m3 out of the east edge.
    s = refstep(oracle_mod, cases.slope(False), fixed=fixed)
    steps = sum(s.advance(10.0)[0] for _ in range(6))
    planes = s.read_state_bits().reshape(4, -1)
    volume = planes[0].astype(np.float64).sum() * 0.25
    led = s.read_ledger()
    pin = PINS["count_of_water_fp32"]
    assert steps == pin["steps"]
    assert round(volume, 5) == pin["volume_m3"]
    assert round(led["open_edge_out_m3"], 4) == pin["open_out_m3"]


def test_fixed_form_reproduces_a_published_device_hash(oracle_mod):
    # The count's flow, 400 steps, Ops::fixed: the reference's Titan Xp log has this hash
    # (water_live.md:43); the fixed form is built from + - x alone, which every IEEE device rounds
    # alike, and the restatement gives the same bytes.
    s = refstep(oracle_mod, cases.slope(False), fixed=True)
    s.run_steps(400, float("inf"))
    assert s.state_hash() == int(PINS["slope_400_fixed_titan_xp"]["hash"])


@pytest.mark.parametrize("name", sorted(k for k in FP64 if not k.startswith("_")))
def test_solver64_reproduces_the_reference_golden_vectors(oracle_mod, name):
    import golden.make_golden as mg
    specs = {n: (c, how) for n, c, how in mg.golden_cases()}
    base = name.replace("_4_workers", "")
    c, how = specs[base]
    workers = 4 if name.endswith("_4_workers") else 1
    g = oracle_mod.Grid(c["nx"], c["ny"], c["cell_m"], open_edges=c.get("open_edges", 0))
    s = oracle_mod.Solver64(g, workers)
    s.set_state(c["h"])
    s.set_inputs(c["bed"], c.get("manning"), c.get("source"))
    if "advance" in how:
        steps = s.advance(how["advance"])
    else:
        for _ in range(how["steps"]):
            s.step(how["max_dt"])
        steps = how["steps"]
    want = FP64[name]
    assert steps == want["steps"]
    assert s.state_hash() == int(want["hash"])
    led = s.ledger()
    assert led["open_edge_out_m3"] == want["open_edge_out_m3"]
    assert led["source_m3"] == want["source_m3"]
    assert led["roundoff_m3"] == want["roundoff_m3"]


@pytest.mark.parametrize("name", ["stoker_400", "ritter_200", "inexact_lake",
                                  "slope_all_open_no_manning", "closed_basin_300_fixed"])
def test_card_form_in_double_equals_the_reference_cpu_tick(oracle_mod, name):
    # The shader's scheme in FP64 (RefStep<double>) is water_state's update, operation for
    # operation: the same bytes as the reference CPU tick on h, hu, hv.
    import golden.make_golden as mg
    c, how = {n: (c, h) for n, c, h in mg.golden_cases()}[name]
    g = oracle_mod.Grid(c["nx"], c["ny"], c["cell_m"], open_edges=c.get("open_edges", 0))
    a = oracle_mod.Solver64(g)
    a.set_state(c["h"])
    a.set_inputs(c["bed"], None, c.get("source"))
    b = refstep(oracle_mod, dict(c, manning=None), precision64=True)
    if "advance" in how:
        assert a.advance(how["advance"]) == b.advance(how["advance"])[0]
    else:
        for _ in range(how["steps"]):
            a.step(how["max_dt"])
        b.run_steps(how["steps"], how["max_dt"])
    A = a.state()
    B = b.read_state_bits().reshape(4, -1)
    for x, y in zip(A, B[:3]):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64))


def test_advance_refuses_a_coarser_source_clock(oracle_mod):
    # water_live.cpp:600-606
    n = 16 * 16
    c = dict(nx=16, ny=16, cell_m=1.0, bed=np.zeros(n), h=np.ones(n), source=np.full(n, -1e-6))
    s = refstep(oracle_mod, c)
    s.set_source(c["source"], every=8)
    steps, refused = s.advance(1.0)
    assert steps == 0 and refused


def test_solver64_thread_count_invariance(oracle_mod):
    # water_state_tests.cpp:739-760: the bytes do not depend on how many threads step the rows.
    c = cases.slope(False)
    hashes = []
    for threads in (1, 3, 8):
        s = oracle_mod.Solver64(oracle_mod.Grid(c["nx"], c["ny"], c["cell_m"], open_edges=2),
                                threads)
        s.set_state(c["h"])
        s.set_inputs(c["bed"], c["manning"], c["source"])
        s.advance(5.0)
        hashes.append(s.state_hash())
    assert hashes[0] == hashes[1] == hashes[2] != 0


def test_prime_of_a_raw_upload_equals_write_state(oracle_mod):
    # The oracle's state event (flush, raw write, prime) leaves the records that write_state's own
    # prime leaves for the same planes: prime_main depends on the state alone.
    c = cases.slope(False)
    a = refstep(oracle_mod, c)
    a.run_steps(30, 0.01)
    planes = a.read_state_bits().copy()
    a.run_length_pass(0.0)
    a.write_planes(planes)
    a.prime()
    b = refstep(oracle_mod, c)
    n = c["nx"] * c["ny"]
    b.write_state(planes[:n].astype(np.float64), planes[n:2 * n].astype(np.float64),
                  planes[2 * n:3 * n].astype(np.float64))
    assert np.array_equal(a.read_partials_bits().view(np.uint32),
                          b.read_partials_bits().view(np.uint32))

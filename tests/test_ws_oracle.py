"""The oracle's complete FP64 step against the reference's own water_state::Solver, compiled from
its sources (oracle/_ref), byte for byte: every state field, every per-cell output, the whole
ledger and the state hash, on cases with the ground store, carried quantities, Manning's friction,
sources, sinks and open edges on. And fdlibm's e^x and ln x as the oracle restates them against the
reference's det::exp and det::log. Skipped where the reference's sources are absent.
"""
from __future__ import annotations

import numpy as np
import pytest

import ws_cases

oracle_mod = pytest.importorskip("oracle")


@pytest.fixture(scope="module")
def both(oracle_mod):
    if not oracle_mod.ref_available() and not oracle_mod.build_ref():
        pytest.skip("the reference's sources are not here")
    return oracle_mod


def make(o, case, reference):
    c = case["config"]
    s = o.FullSolver(c["nx"], c["ny"], c["cell_m"], open_edges=c["open_edges"],
                     carried=c["carried"], reference=reference)
    ws_cases.load(s, case)
    return s


@pytest.mark.parametrize("name", sorted(ws_cases.CASES))
def test_full_step_equals_the_reference(both, name):
    case = ws_cases.CASES[name]()
    a, b = make(both, case, False), make(both, case, True)
    ra, rb = ws_cases.run(a, case), ws_cases.run(b, case)
    assert ra == rb
    for f in ws_cases.FIELDS:
        x, y = a.get(f), b.get(f)
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64)), (name, f)
    la, lb = a.ledger(), b.ledger()
    assert la == lb, name
    assert a.state_hash() == b.state_hash()
    # Every part of the step did something in the case.
    if case["config"]["carried"]:
        assert np.abs(a.get("carried")).max() > 0
    if "ground_k" in case["inputs"]:
        assert la["ground_m3"] > 0


def test_fdlibm_exp_and_log_equal_the_reference(both):
    rng = np.random.default_rng(17)
    x = np.concatenate([rng.uniform(-745, 710, 300000), rng.uniform(-1, 1, 300000),
                        rng.uniform(-1e-7, 1e-7, 10000), -np.abs(rng.standard_normal(10000)) / 30,
                        [0.0, -0.0, 1e-300, -1e-300, 709.78, -745.1, np.inf, -np.inf, np.nan]])
    a, b = both.fd_exp(x), both.ref_det("exp", x)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    y = np.concatenate([np.exp(rng.uniform(-700, 700, 300000)), rng.uniform(0.5, 2, 300000),
                        1 + rng.uniform(-1e-6, 1e-6, 10000), rng.uniform(1e-9, 100, 100000),
                        [1.0, 5e-324, 1e-310, 2.0, 0.0, -1.0, np.inf, np.nan]])
    a, b = both.fd_log(y), both.ref_det("log", y)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def digest(a):
    h = 0xcbf29ce484222325
    for byte in np.ascontiguousarray(a, dtype=np.float64).tobytes():
        h ^= byte
        h = (h * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return f"{h:016x}"


def full_pins():
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    return json.load(open(os.path.join(here, "golden", "ws_full_pins.json")))


@pytest.mark.parametrize("name", sorted(ws_cases.CASES))
def test_oracle_matches_the_reference_pins(oracle_mod, name):
    """The committed pins (tests/golden/make_ws_pins.py, from the reference's own build): the
    oracle's restatement reproduces them wherever it runs."""
    pin = full_pins()[name]
    case = ws_cases.CASES[name]()
    s = make(oracle_mod, case, False)
    assert [float(r) for r in ws_cases.run(s, case)] == pin["results"]
    assert str(s.state_hash()) == pin["state_hash"]
    for f in ws_cases.FIELDS:
        assert digest(s.get(f)) == pin["outputs"][f], f
    led = s.ledger()
    assert {k: float(v) for k, v in led.items() if k != "carried"} == pin["ledger"]
    assert [{k: float(v) for k, v in d.items()} for d in led["carried"]] == pin["carried_ledger"]

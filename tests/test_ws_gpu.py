"""The complete FP64 step on the device (water_state::Solver: ground store, carried quantities,
per-cell outputs, the whole ledger) against the oracle's restatement, which is itself pinned to
the reference's own build (tests/test_ws_oracle.py), byte for byte: every field, every output,
the ledger, the state hash and each call's result. Also against the reference's committed pins,
from a captured graph of steps, and on a larger grid with everything on.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

import oracle
import ws_cases
from game_engine_gb300 import water_state as ws

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def device_solver(case):
    c = case["config"]
    e = c["open_edges"]
    s = ws.Solver(ws.Config(c["nx"], c["ny"], c["cell_m"], carried=list(c["carried"]),
                            west_open=bool(e & 1), east_open=bool(e & 2), south_open=bool(e & 4),
                            north_open=bool(e & 8)))
    ws_cases.load(s, case)
    return s


def oracle_solver(case):
    c = case["config"]
    s = oracle.FullSolver(c["nx"], c["ny"], c["cell_m"], open_edges=c["open_edges"],
                          carried=c["carried"])
    ws_cases.load(s, case)
    return s


def assert_same(dev, ref, what):
    for f in ws_cases.FIELDS:
        a, b = dev.get(f), ref.get(f)
        diff = np.nonzero(a.view(np.uint64) != b.view(np.uint64))[0]
        assert diff.size == 0, f"{what}: {f}: {diff.size} differ, first at {diff[:4]}"
    la, lb = dev.ledger(), ref.ledger()
    for k in oracle.LEDGER_KEYS:
        assert la[k] == lb[k], (what, k, la[k], lb[k])
    for qa, qb in zip(la["carried"], lb["carried"]):
        for k in oracle.CARRIED_LEDGER_KEYS:
            assert qa[k] == qb[k], (what, "carried", k)
    assert dev.state_hash() == ref.state_hash()


@pytest.mark.parametrize("name", sorted(ws_cases.CASES))
def test_full_step_equals_the_oracle(gpu, name):
    case = ws_cases.CASES[name]()
    dev, ref = device_solver(case), oracle_solver(case)
    assert ws_cases.run(dev, case) == ws_cases.run(ref, case)
    assert_same(dev, ref, name)
    pin = json.load(open(os.path.join(HERE, "golden", "ws_full_pins.json")))[name]
    assert str(dev.state_hash()) == pin["state_hash"]
    dev.close()


def test_stable_step_volumes_and_reset(gpu):
    case = ws_cases.slope_full()
    dev, ref = device_solver(case), oracle_solver(case)
    ws_cases.run(dev, case)
    ws_cases.run(ref, case)
    stable = dev.stable_step()
    assert stable > 0 and np.isfinite(stable)
    h = ref.get("depth")
    cell_area = case["config"]["cell_m"] ** 2
    want = 0.0
    for v in h:  # the reference's index-order sum
        want += v
    assert dev.surface_volume_m3() == want * cell_area
    dev.reset_ledger()
    led = dev.ledger()
    assert led["steps"] == 0 and led["time_s"] == 0.0 and led["source_m3"] == 0.0
    dev.close()


def test_inputs_that_do_not_fit_change_nothing(gpu):
    case = ws_cases.slope_full()
    dev = device_solver(case)
    inputs = dict(case["inputs"])
    inputs["ground_s"] = None  # the ground's three spans: all or none (water_state.cpp:156-162)
    h = dev.state_hash()
    assert dev.step(inputs, 0.01) == 0.0 and dev.advance(inputs, 1.0) == 0
    assert dev.state_hash() == h
    assert dev.step(case["inputs"], -1.0) == 0.0
    dev.close()


def test_steps_from_a_captured_graph(gpu):
    import torch
    case = ws_cases.basin_full()
    dev, ref = device_solver(case), oracle_solver(case)
    dev.set_inputs(case["inputs"])
    stream = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        assert dev.enqueue_steps(torch.cuda.current_stream().cuda_stream, 5, 0.004)
    for _ in range(6):
        graph.replay()
        for _ in range(5):
            ref.step(case["inputs"], 0.004)
    torch.cuda.synchronize()
    assert_same(dev, ref, "graph")
    dev.close()


def test_a_larger_grid_with_everything_on(gpu):
    """320 x 288 (odd multiples), fBm relief, every input on, 40 steps, against the oracle."""
    from game_engine_gb300 import workloads
    nx, ny = 320, 288
    n = nx * ny
    rng = np.random.default_rng(9)
    bed = workloads.fbm(nx, ny, 3.0, 1234)
    h = np.maximum(1.5 + 0.1 * rng.standard_normal(n) - bed, 0.0)
    case = dict(config=dict(nx=nx, ny=ny, cell_m=1.0, open_edges=5,
                            carried=[(20.0, 2e-4, 0.1), (0.0, 0.0, 0.0), (5.0, 0.0, 0.0)]),
                fields=dict(depth=h, momentum_x=0.05 * rng.standard_normal(n),
                            momentum_y=0.05 * rng.standard_normal(n),
                            ground=np.full(n, 0.01),
                            carried=np.concatenate([np.zeros(n), np.full(n, 0.02) * (h > 0),
                                                    np.full(n, 0.1) * (h > 0)])),
                inputs=dict(bed=bed, manning=np.full(n, 0.025), source=np.full(n, 2e-5),
                            ground_k=np.full(n, 5e-6), ground_s=np.full(n, 0.08),
                            ground_cap=np.full(n, 0.1),
                            carried_source=[None, np.full(n, 1e-6), None],
                            carried_exchange=[None, -1e-5 * (1 + rng.random(n)), None]),
                run=[("step", 0.05)] * 40)
    dev, ref = device_solver(case), oracle_solver(case)
    assert ws_cases.run(dev, case) == ws_cases.run(ref, case)
    assert_same(dev, ref, "320x288")
    dev.close()


def test_the_benchmark_configuration_first_steps(gpu):
    """The full_step benchmark's 2048 x 2048 tile with every input on: its first 3 steps against
    the oracle, byte for byte (the oracle takes about a second a step)."""
    from game_engine_gb300 import workloads
    t, config, fields, inputs = workloads.full_step(2048)
    case = dict(config=dict(config, open_edges=0), fields=fields, inputs=inputs,
                run=[("step", 0.01)] * 3)
    dev, ref = device_solver(case), oracle_solver(case)
    assert ws_cases.run(dev, case) == ws_cases.run(ref, case)
    assert_same(dev, ref, "2048")
    dev.close()


@pytest.mark.parametrize("nx,ny,edges", [(1, 1, 15), (1, 37, 3), (45, 3, 12), (17, 33, 5),
                                         (64, 1, 0)])
def test_odd_and_degenerate_grids(gpu, nx, ny, edges):
    """Single cells, single rows and columns, odd sizes, every edge combination, everything on."""
    n = nx * ny
    rng = np.random.default_rng(nx * 1000 + ny)
    bed = rng.uniform(0.0, 0.3, n)
    case = dict(config=dict(nx=nx, ny=ny, cell_m=0.5, open_edges=edges,
                            carried=[(3.0, 1e-3, 0.0), (0.0, 0.0, 0.0)]),
                fields=dict(depth=rng.uniform(0.0, 0.4, n), momentum_x=0.02 * rng.standard_normal(n),
                            momentum_y=0.02 * rng.standard_normal(n), ground=np.zeros(n),
                            carried=np.concatenate([np.zeros(n), rng.uniform(0, 0.01, n)])),
                inputs=dict(bed=bed, manning=np.full(n, 0.02), source=rng.uniform(-1e-3, 1e-3, n),
                            ground_k=np.full(n, 1e-5), ground_s=np.full(n, 0.05),
                            ground_cap=np.full(n, 0.02),
                            carried_source=[None, None],
                            carried_exchange=[None, rng.uniform(-2e-4, 1e-4, n)]),
                run=[("step", 0.02), ("advance", 0.5)])
    dev, ref = device_solver(case), oracle_solver(case)
    assert ws_cases.run(dev, case) == ws_cases.run(ref, case)
    assert_same(dev, ref, f"{nx}x{ny}")
    dev.close()

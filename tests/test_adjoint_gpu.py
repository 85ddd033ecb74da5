"""The adjoint on the device (wl_adjoint_*): its forward ticks are the plain tick to the bit, its
gradients are the oracle's reverse sweep and the FP64 replay's central differences within 1e-4
(the largest error over the largest magnitude), they do not depend on the checkpoint interval, the
graph, or the batch a tile sits in, and the sweep refuses what it does not differentiate.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

import oracle
from adjoint_cases import basin, fd_cells, grid, probes_and_targets, rel_err
from game_engine_gb300 import water_live as wl
from game_engine_gb300 import workloads
from game_engine_gb300.adjoint import Adjoint, AdjointError
from game_engine_gb300.batch import Batch
from pairs import config

pytestmark = pytest.mark.gpu

DT = 0.01
TOL = 1e-4
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def device_step(c, source=True, fixed=False):
    dev = wl.DeviceStep()
    ok = dev.create(config(c), wl.StepOptions(ops=wl.OPS_FIXED if fixed else wl.OPS_NATIVE))
    assert ok, dev.error
    assert dev.set_bed(c["bed"]), dev.error
    if source:
        assert dev.set_source(c["source"]), dev.error
    n = c["nx"] * c["ny"]
    assert dev.write_state(c["h"], np.zeros(n), np.zeros(n)), dev.error
    return dev


@pytest.mark.parametrize("edges,sinks", [(0, False), (15, False), (9, True)])
def test_sweep_forward_is_the_plain_tick(gpu, edges, sinks):
    c = basin(70, 45, 3, edges=edges, sinks=sinks)  # partial bands and rows
    ticks = 60
    dev = device_step(c)
    probes, targets = probes_and_targets(c, ticks, DT, 6, seed=1)
    a = Adjoint(dev, ticks, 7, probes, targets)
    a.run(DT)
    fin = a.read_final().reshape(3, -1)
    _, _, _, limited = a.read()
    assert limited[0] == 0
    want, _ = oracle.adj_forward(grid(c), DT, ticks, c["bed"], c["source"], c["state0"])
    assert np.array_equal(bits(fin), bits(want.astype(np.float32)))
    h0 = dev.state_hash()
    dev.run_steps(ticks, DT)  # the plain tick from the same state: the sweep left it alone
    plain = dev.read_state_bits().reshape(4, -1)[:3]
    assert np.array_equal(bits(fin), bits(plain))
    assert h0 != dev.state_hash()
    a.close()


@pytest.mark.parametrize("edges,seed,sinks", [(0, 7, False), (15, 8, False), (6, 9, True)])
def test_gradients_are_the_oracle_sweep(gpu, edges, seed, sinks):
    c = basin(24, 20, seed, edges=edges, sinks=sinks)
    ticks = 120
    probes, targets = probes_and_targets(c, ticks, DT, 12, seed=seed)
    dev = device_step(c)
    a = Adjoint(dev, ticks, 16, probes, targets)
    a.run(DT)
    loss, g_bed, g_src, limited = a.read()
    assert limited[0] == 0
    args = (grid(c), DT, ticks, c["bed"], c["source"], c["state0"], probes, targets)
    l32, b32, s32, _ = oracle.adjoint(*args, precision64=False)
    l64, b64, s64, _ = oracle.adjoint(*args, precision64=True)
    assert loss[0] == pytest.approx(l32, rel=1e-12)  # the same FP32 depths, the loss in FP64
    assert rel_err(g_bed, b32) < 1e-5 and rel_err(g_src, s32) < 1e-5
    assert rel_err(g_bed, b64) < TOL and rel_err(g_src, s64) < TOL
    cells = fd_cells(c, 16, seed=5, eps=1e-3)
    fd_bed, fd_src = oracle.adj_fd(*args, cells, eps_bed=1e-3, rel_source=1e-3)
    assert rel_err(g_bed[cells], fd_bed) < TOL
    assert rel_err(g_src[cells], fd_src) < TOL
    if sinks:
        assert np.count_nonzero(a.read_final()[: c["nx"] * c["ny"]] == 0.0) > 0
    a.close()


@pytest.mark.parametrize("edges,seed,sinks", [(0, 7, False), (6, 9, True)])
def test_the_starting_state_gradient_is_the_oracle_sweep(gpu, edges, seed, sinks):
    """dL/d(h0, hu0, hv0) read back after the sweep: the oracle's FP32 sweep within 1e-5, its
    FP64 sweep (pinned to the FP64 replay's central differences on the CPU) within 1e-4."""
    c = basin(24, 20, seed, edges=edges, sinks=sinks)
    ticks = 120
    probes, targets = probes_and_targets(c, ticks, DT, 12, seed=seed)
    dev = device_step(c)
    a = Adjoint(dev, ticks, 16, probes, targets)
    a.run(DT)
    lam = a.read_state_gradient()
    args = (grid(c), DT, ticks, c["bed"], c["source"], c["state0"], probes, targets)
    *_, g32 = oracle.adjoint(*args, precision64=False, state_gradient=True)
    *_, g64 = oracle.adjoint(*args, precision64=True, state_gradient=True)
    assert rel_err(lam, g32) < 1e-5
    assert rel_err(lam, g64) < TOL
    # a second sweep from the same state gives the same bytes
    a.run(DT, graph=True)
    assert np.array_equal(bits(a.read_state_gradient()), bits(lam))
    a.close()


def test_checkpoint_interval_graph_and_replay_change_no_byte(gpu):
    c = basin(50, 37, 4, edges=5, sinks=True)
    ticks = 45
    probes, targets = probes_and_targets(c, ticks, DT, 9, seed=3)
    dev = device_step(c)
    results = []
    for every, graph in ((1, True), (4, False), (4, True), (45, True), (100, False)):
        a = Adjoint(dev, ticks, every, probes, targets)
        a.run(DT, graph=graph)
        if graph:
            a.run(DT, graph=True)  # a replay of the captured sweep
        results.append(a.read())
        a.close()
    for r in results[1:]:
        for got, want in zip(r, results[0]):
            assert np.array_equal(np.asarray(got).view(np.uint8), np.asarray(want).view(np.uint8))


def test_a_batch_sweep_is_each_tile_swept_alone(gpu):
    specs = [(40, 31, 0, 11), (17, 64, 15, 12), (96, 33, 6, 13), (5, 7, 0, 14)]
    ticks, every = 30, 8
    tiles, probes, targets, alone = [], [], [], []
    for nx, ny, edges, seed in specs:
        c = basin(nx, ny, seed, edges=edges, sinks=(seed == 13))
        p, t = probes_and_targets(c, ticks, DT, min(5, nx * ny), seed=seed)
        dev = device_step(c)
        a = Adjoint(dev, ticks, every, p, t)
        a.run(DT)
        alone.append(a.read() + (a.read_final(), a.read_state_gradient()))
        a.close()
        tiles.append(c)
        probes.append(p)
        targets.append(t)
    b = Batch([(c["nx"], c["ny"]) for c in tiles], open_edges=[c["open_edges"] for c in tiles])
    b.set_bed(np.concatenate([c["bed"] for c in tiles]))
    b.set_source(np.concatenate([c["source"] for c in tiles]))
    b.write_state(np.concatenate([c["h"] for c in tiles]))
    a = Adjoint(b, ticks, every, probes, targets)
    a.run(DT)
    loss, g_bed, g_src, limited = a.read()
    fin = a.read_final()
    lam = a.read_state_gradient()
    first, first3 = 0, 0
    for k, c in enumerate(tiles):
        n = c["nx"] * c["ny"]
        l1, gb1, gs1, lim1, fin1, lam1 = alone[k]
        assert loss[k] == l1[0] and limited[k] == lim1[0]
        assert np.array_equal(g_bed[first:first + n], gb1)
        assert np.array_equal(g_src[first:first + n], gs1)
        assert np.array_equal(bits(fin[first3:first3 + 3 * n]), bits(fin1))
        assert np.array_equal(bits(lam[first3:first3 + 3 * n]), bits(lam1))
        first += n
        first3 += 3 * n
    a.close()
    b.close()


def test_the_sweep_refuses_what_it_does_not_differentiate(gpu):
    c = basin(20, 16, 2)
    probes, targets = np.array([5], np.uint32), np.array([1.0])
    dev = device_step(c, fixed=True)
    with pytest.raises(AdjointError, match="native"):
        Adjoint(dev, 10, 5, probes, targets)
    dev = device_step(c)
    a = Adjoint(dev, 10, 5, probes, targets)
    assert dev.set_manning(np.full(c["nx"] * c["ny"], 0.03))
    with pytest.raises(AdjointError, match="Manning"):
        a.run(DT)
    a.close()
    dev = device_step(c, source=False)
    assert dev.set_source(c["source"], every=3)
    with pytest.raises(AdjointError, match="every step"):
        Adjoint(dev, 10, 5, probes, targets)
    dev = device_step(c)
    with pytest.raises(AdjointError, match="outside"):
        Adjoint(dev, 10, 5, np.array([c["nx"] * c["ny"]], np.uint32), targets)
    with pytest.raises(AdjointError, match="ticks > 0"):
        Adjoint(dev, 0, 5, probes, targets)


def test_repeated_probes_and_a_single_tick(gpu):
    # A probe listed twice counts twice (the loss and the seed add in probe order); T = 1 and
    # k = 1 are the smallest sweep.
    c = basin(30, 22, 6, edges=10)
    for ticks, every in ((1, 1), (9, 2)):
        probes = np.array([7, 7, 100, 651], np.uint32)
        fin, _ = oracle.adj_forward(grid(c), DT, ticks, c["bed"], c["source"], c["state0"],
                                    precision64=True)
        targets = fin[0][probes] + np.array([0.01, -0.02, 0.03, 0.0])
        dev = device_step(c)
        a = Adjoint(dev, ticks, every, probes, targets)
        a.run(DT)
        loss, g_bed, g_src, limited = a.read()
        l32, b32, s32, _ = oracle.adjoint(grid(c), DT, ticks, c["bed"], c["source"],
                                          c["state0"], probes, targets, precision64=False)
        assert limited[0] == 0
        assert loss[0] == pytest.approx(l32, rel=1e-12)
        assert rel_err(g_bed, b32) < 1e-5 and rel_err(g_src, s32) < 1e-5
        a.close()


def test_shortened_ticks_are_counted(gpu):
    c = basin(20, 16, 1, level=30.0)
    dev = device_step(c)
    a = Adjoint(dev, 10, 4, np.array([3], np.uint32), np.array([1.0]))
    a.run(0.05)
    _, _, _, limited = a.read()
    _, want = oracle.adj_forward(grid(c), 0.05, 10, c["bed"], c["source"], c["state0"])
    assert limited[0] == want == 10
    a.close()


def test_adjoint_configuration_against_central_differences(gpu):
    """The full adjoint configuration (512 x 512, 2000 ticks, a checkpoint every 50, 64 probes)
    against the FP64 replay's central differences at 32 cells (tests/golden/adjoint_512_fd.json,
    made by make_adjoint_fd.py)."""
    with open(os.path.join(GOLDEN, "adjoint_512_fd.json")) as f:
        fd = json.load(f)
    t = workloads.adjoint_512()
    assert (t.nx, t.ny, t.meta["ticks"], t.meta["every"]) == (fd["nx"], fd["ny"], fd["ticks"],
                                                             fd["every"])
    dev = wl.DeviceStep()
    assert dev.create(wl.Config(t.nx, t.ny, t.cell_m)), dev.error
    assert dev.set_bed(t.bed) and dev.set_source(t.source)
    assert dev.write_state(t.h, t.hu, t.hv)
    a = Adjoint(dev, fd["ticks"], fd["every"], fd["probes"], fd["targets"])
    a.run(fd["max_dt"])
    loss, g_bed, g_src, limited = a.read()
    assert limited[0] == 0
    assert loss[0] == pytest.approx(fd["loss_fp64"], rel=1e-3)
    cells = np.array(fd["fd_cells"])
    err_bed = rel_err(g_bed[cells], fd["fd_bed"])
    err_src = rel_err(g_src[cells], fd["fd_source"])
    print(f"adjoint_512: bed {err_bed:.2e}, source {err_src:.2e} (max-norm relative, "
          f"{cells.size} cells)")
    assert err_bed < TOL
    assert err_src < TOL
    # the sweep's tick-2000 state is the plain tick's
    fin = a.read_final().reshape(3, -1)
    dev.run_steps(fd["ticks"], fd["max_dt"])
    assert np.array_equal(bits(fin), bits(dev.read_state_bits().reshape(4, -1)[:3]))
    a.close()

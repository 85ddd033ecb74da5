"""The adjoint's oracle (oracle/wl_adjoint.hpp), on the CPU: its forward is the card's step to the
bit, and its FP64 reverse sweep is the gradient of the FP64 replay (central differences)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from adjoint_cases import basin, fd_cells, grid, probes_and_targets, rel_err

DT = 0.01


@pytest.mark.parametrize("edges,sinks", [(0, False), (15, False), (5, True)])
def test_fixed_step_forward_is_the_card_step(oracle_mod, edges, sinks):
    c = basin(40, 28, 3, edges=edges, sinks=sinks)
    ticks = 60
    got, limited = oracle.adj_forward(grid(c), DT, ticks, c["bed"], c["source"], c["state0"])
    assert limited == 0
    r = oracle.RefStep(grid(c))
    r.set_bed(c["bed"])
    r.set_source(c["source"])
    n = c["nx"] * c["ny"]
    r.write_state(c["h"], np.zeros(n), np.zeros(n))
    r.run_steps(ticks, DT)
    want = r.read_state_bits().reshape(4, -1)[:3]
    assert np.array_equal(got.astype(np.float32).view(np.uint32), want.view(np.uint32))
    if sinks:
        assert np.count_nonzero(got[0] == 0.0) > 0  # the sinks dried cells


def test_shortened_ticks_are_counted(oracle_mod):
    c = basin(20, 16, 1, level=30.0)
    _, limited = oracle.adj_forward(grid(c), 0.05, 10, c["bed"], c["source"], c["state0"])
    assert limited == 10


@pytest.mark.parametrize("edges,seed", [(0, 7), (15, 8), (6, 9)])
def test_fp64_sweep_is_the_fp64_replay_gradient(oracle_mod, edges, seed):
    c = basin(24, 20, seed, edges=edges)
    ticks = 120
    probes, targets = probes_and_targets(c, ticks, DT, 12, seed=seed)
    loss, g_bed, g_src, limited = oracle.adjoint(grid(c), DT, ticks, c["bed"], c["source"],
                                                 c["state0"], probes, targets)
    assert limited == 0 and loss > 0
    assert loss == pytest.approx(oracle.adj_loss64(grid(c), DT, ticks, c["bed"], c["source"],
                                                   c["state0"], probes, targets), rel=1e-12)
    cells = fd_cells(c, 16, seed=5, eps=1e-3)
    fd_bed, fd_src = oracle.adj_fd(grid(c), DT, ticks, c["bed"], c["source"], c["state0"], probes,
                                   targets, cells, eps_bed=1e-3, rel_source=1e-3)
    assert rel_err(g_bed[cells], fd_bed) < 1e-4
    assert rel_err(g_src[cells], fd_src) < 1e-4


def test_a_bed_tie_is_a_kink(oracle_mod):
    # Where a cell's bed ties a neighbour's within the difference's half-width, the central
    # difference straddles the reconstruction's kink and is not the derivative: the reason the
    # difference cells are drawn away from ties.
    c = basin(24, 20, 7)
    ticks = 120
    probes, targets = probes_and_targets(c, ticks, DT, 12, seed=7)
    _, g_bed, _, _ = oracle.adjoint(grid(c), DT, ticks, c["bed"], c["source"], c["state0"],
                                    probes, targets)
    k = 463  # (7, 19): its east neighbour's bed is 4.6e-5 m above its own
    assert 0 < c["bed"][k + 1] - c["bed"][k] < 1e-4
    args = (grid(c), DT, ticks, c["bed"], c["source"], c["state0"], probes, targets, [k])
    near, _ = oracle.adj_fd(*args, eps_bed=1e-5)
    across, _ = oracle.adj_fd(*args, eps_bed=1e-3)
    assert rel_err(g_bed[[k]], near) < 1e-5
    assert rel_err(g_bed[[k]], across) > 1e-4


def test_fp32_sweep_is_close_to_the_fp64_sweep(oracle_mod):
    c = basin(24, 20, 9, edges=3)
    ticks = 120
    probes, targets = probes_and_targets(c, ticks, DT, 12, seed=2)
    args = (grid(c), DT, ticks, c["bed"], c["source"], c["state0"], probes, targets)
    l64, b64, s64, _ = oracle.adjoint(*args, precision64=True)
    l32, b32, s32, _ = oracle.adjoint(*args, precision64=False)
    assert l32 == pytest.approx(l64, rel=1e-4)
    assert rel_err(b32, b64) < 1e-4
    assert rel_err(s32, s64) < 1e-4


def state_fd(c, ticks, probes, targets, cells, eps=1e-4):
    """Central differences of the FP64 replay's loss on each of the three starting planes at
    `cells`, plane after plane."""
    n = c["nx"] * c["ny"]
    args = (grid(c), DT, ticks, c["bed"], c["source"])
    out = []
    for plane in range(3):
        for k in cells:
            s0 = np.array(c["state0"], dtype=np.float64)
            s0[plane * n + k] += eps
            up = oracle.adj_loss64(*args, s0, probes, targets)
            s0[plane * n + k] -= 2 * eps
            down = oracle.adj_loss64(*args, s0, probes, targets)
            out.append((up - down) / (2 * eps))
    return np.array(out)


def wet_cells(c, count, seed, depth=0.3):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(np.nonzero(c["h"] > depth)[0], size=count, replace=False))


@pytest.mark.parametrize("edges,seed", [(0, 7), (15, 8)])
def test_the_starting_state_gradient_is_the_fp64_replay_gradient(oracle_mod, edges, seed):
    """dL/d(h0, hu0, hv0), the FP64 sweep's adjoint state after its last reverse tick, against
    central differences of the FP64 replay at wet cells; the FP32 sweep's within 1e-4 of it."""
    c = basin(24, 20, seed, edges=edges)
    ticks = 120
    probes, targets = probes_and_targets(c, ticks, DT, 12, seed=seed)
    args = (grid(c), DT, ticks, c["bed"], c["source"], c["state0"], probes, targets)
    *_, g64 = oracle.adjoint(*args, state_gradient=True)
    *_, g32 = oracle.adjoint(*args, precision64=False, state_gradient=True)
    n = c["nx"] * c["ny"]
    cells = wet_cells(c, 8, seed=3)
    fd = state_fd(c, ticks, probes, targets, cells)
    got = np.concatenate([g64[p * n + cells] for p in range(3)])
    assert rel_err(got, fd) < 1e-4
    assert rel_err(g32, g64) < 1e-4

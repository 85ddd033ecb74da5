"""The benchmark configurations themselves, at full size, against the oracle's answers in
tests/golden/configs.json (written by tests/golden/make_configs.py from the oracle's FP32
restatement of the card's step, on the CPU):

  - the 2048 x 2048 throughput tile after its 500 ticks: the state hash, each plane's hash, the
    ledger's bits and the records' hash;
  - the 4096-tile batch after its 200 ticks, in the shape the autotuner chooses: every tile's hash;
  - the 256-tile batched adjoint (500 ticks, a checkpoint every 25): each tile's loss, and its
    gradients with respect to the bed and the source at its 64 probes and 32 seeded cells, within
    1e-5 of the tile's largest gradient (the reverse sweep's derivative-only arithmetic takes
    fast reciprocals and contraction; its forward is bit-exact); and on four tiles, against the
    FP64 replay's central differences within 1e-4.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from game_engine_gb300 import water_live as wl, workloads

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "configs.json")
ADJOINT_TOL = 1e-5
FD_TOL = 1e-4


def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def test_plain_2048_after_500_ticks(gpu):
    g = golden()["plain_2048"]
    t = workloads.plain_2048()
    dev = wl.DeviceStep()
    assert dev.create(wl.Config(t.nx, t.ny, t.cell_m)), dev.error
    assert dev.set_bed(t.bed) and dev.set_source(t.source)
    assert dev.write_state(t.h, t.hu, t.hv), dev.error
    assert dev.run_steps(g["ticks"], g["max_dt"]), dev.error
    import oracle
    planes = dev.read_state_bits().reshape(4, -1)
    assert [oracle.hash_floats(p) for p in planes] == g["plane_hashes"]
    assert dev.state_hash() == g["hash"]
    assert [int(v) for v in dev.read_ledger_bits()] == g["ledger_bits"]
    assert oracle.hash_floats(dev.read_partials_bits().ravel()) == g["records_hash"]
    dev.destroy()


def test_tiles_4096_after_200_ticks(gpu):
    from game_engine_gb300.batch import Batch, concat
    g = golden()["tiles_4096"]
    tiles = workloads.tiles_4096(g["count"])
    b = Batch([(t.nx, t.ny) for t in tiles])
    b.set_bed(concat(tiles, "bed"))
    b.write_state(concat(tiles, "h"))
    del tiles
    b.autotune(g["max_dt"], trial_ticks=2)
    b.run_ticks(g["ticks"], g["max_dt"], graph=True)
    got = [int(h) for h in b.tile_hashes()]
    bad = [k for k, (a, w) in enumerate(zip(got, g["hashes"])) if a != w]
    assert not bad, f"{len(bad)} tiles differ, first {bad[:8]} (tuning {b.tuning()})"
    b.close()


def test_tiles_256_adjoint_losses_and_gradients(gpu):
    from game_engine_gb300.adjoint import Adjoint
    from game_engine_gb300.batch import Batch, concat
    g = golden()["tiles_256_adjoint"]
    tiles = workloads.tiles_256_adjoint(g["count"])
    sides = [(t.nx, t.ny) for t in tiles]
    b = Batch(sides)
    b.set_bed(concat(tiles, "bed"))
    b.set_source(concat(tiles, "source"))
    b.write_state(concat(tiles, "h"))
    probes = [t.meta["probes"] for t in tiles]
    targets = [np.array(r["targets"]) for r in g["tiles"]]
    a = Adjoint(b, g["ticks"], g["every"], probes, targets)
    a.run(g["max_dt"])
    loss, g_bed, g_src, limited = a.read()
    assert int(limited.sum()) == 0
    worst = 0.0
    for k, r in enumerate(g["tiles"]):
        sl = b.tile_slice(k)
        assert loss[k] == pytest.approx(r["loss"], rel=1e-6, abs=1e-12), k
        for key, grad, scale in (("g_bed", g_bed[sl], r["g_bed_max"]),
                                 ("g_src", g_src[sl], r["g_src_max"])):
            for where, cells in (("probes", probes[k]), ("cells", np.array(r["cells"]))):
                want = np.array(r[f"{key}_{where}"])
                err = float(np.max(np.abs(grad[cells] - want))) / max(scale, 1e-300)
                worst = max(worst, err)
                assert err < ADJOINT_TOL, (k, key, where, err)
    print(f"tiles_256_adjoint: worst gradient error {worst:.2e} of each tile's largest")
    # Against the FP64 replay's central differences on four tiles (the adjoint's bound, 1e-4 of
    # the largest difference at the tile's cells).
    from adjoint_cases import rel_err
    for r in golden()["tiles_256_adjoint_fd"]:
        k = r["index"]
        sl = b.tile_slice(k)
        cells = np.array(r["cells"])
        assert loss[k] == pytest.approx(r["loss_fp64"], rel=1e-3), k
        err_bed = rel_err(g_bed[sl][cells], r["fd_bed"])
        err_src = rel_err(g_src[sl][cells], r["fd_src"])
        print(f"tile {k} ({r['nx']}x{r['ny']}): bed {err_bed:.2e}, source {err_src:.2e} of FD")
        assert err_bed < FD_TOL and err_src < FD_TOL, (k, err_bed, err_src)
    a.close()
    b.close()

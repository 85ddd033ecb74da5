"""Writes tests/golden/configs.json: the oracle's answers on the benchmark configurations at their
full sizes, so that the GPU tests (and bench.py, after its timed run) hold the timed workloads
themselves to the oracle, not only smaller cases of the same code:

  plain_2048         the FP32 restatement of the card's step (oracle RefStep<float>) on the
                     2048 x 2048 throughput tile, 500 ticks of max_dt 0.01 s with rain: the state
                     hash (FNV-1a over the four planes, water_live.cpp:90-101), each plane's hash,
                     the ledger's bits and the records' hash;
  tiles_4096         the 4096 uneven tiles, 200 ticks each: every tile's state hash;
  tiles_256_adjoint  the batched adjoint configuration (256 tiles, 500 ticks): each tile's targets
                     from the oracle's FP32 run on the perturbed bed, then the oracle's FP32
                     reverse sweep: the loss, and the gradients with respect to the bed and the
                     source at the tile's 64 probe cells and at 32 seeded cells, with each
                     gradient's largest magnitude;
  tiles_256_adjoint_fd  for four of those tiles (sides 64, 128, 192 and 256), central differences
                     of the FP64 replay's loss at 8 cells each, on the bed (eps 1e-3 m) and the
                     source (1e-3 relative), at cells drawn away from bed ties.

Terrain comes from workloads.fbm_numpy (the same doubles as the library's generator), so nothing
here loads the CUDA library. Work is dealt to processes (spawn) by tile, each building only the
tiles it steps. About 25 minutes on 8 cores.

    python tests/golden/make_configs.py [--only plain_2048,tiles_4096,tiles_256_adjoint]
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

OUT = os.path.join(HERE, "configs.json")
GRAD_CELLS = 32


def _plain_2048():
    import oracle
    from game_engine_gb300 import workloads as W
    t = W.plain_2048(terrain=W.fbm_numpy)
    r = oracle.RefStep(oracle.Grid(t.nx, t.ny, t.cell_m))
    r.set_bed(t.bed)
    r.set_source(t.source)
    r.write_state(t.h, t.hu, t.hv)
    ticks, max_dt = t.meta["ticks"], t.meta["max_dt"]
    r.run_steps(ticks, max_dt)
    planes = r.read_state_bits().reshape(4, -1)
    return dict(nx=t.nx, ny=t.ny, ticks=ticks, max_dt=max_dt, hash=r.state_hash(),
                plane_hashes=[oracle.hash_floats(p) for p in planes],
                ledger_bits=[int(v) for v in r.read_ledger_bits()],
                records_hash=oracle.hash_floats(r.read_partials_bits().ravel()),
                steps=r.read_ledger()["steps"])


def _tiles_4096_part(args):
    first, last = args
    import oracle
    from game_engine_gb300 import workloads as W
    tiles = W.tiles_4096(terrain=W.fbm_numpy, only=range(first, last))
    out = []
    for k in range(first, last):
        t = tiles[k]
        r = oracle.RefStep(oracle.Grid(t.nx, t.ny, t.cell_m))
        r.set_bed(t.bed)
        r.write_state(t.h, t.hu, t.hv)
        r.run_steps(200, W.MAX_DT)
        out.append(r.state_hash())
    return first, out


def _adjoint_tile(k):
    import oracle
    from game_engine_gb300 import workloads as W
    t = W.tiles_256_adjoint(terrain=W.fbm_numpy, only=[k])[k]
    seed = W.SEEDS["tiles_256_adjoint"]
    ticks, dt = W.TILES_ADJOINT_TICKS, W.MAX_DT
    g = oracle.Grid(t.nx, t.ny, t.cell_m)
    # The targets: the FP32 tick on the perturbed bed (the device's target run), probe depths.
    tgt = oracle.RefStep(g)
    tgt.set_bed(W.perturbed_bed(t.bed, seed + k))
    tgt.set_source(t.source)
    tgt.write_state(t.h, t.hu, t.hv)
    tgt.run_steps(ticks, dt)
    probes = t.meta["probes"]
    targets = tgt.read_state_bits()[:t.cells][probes].astype(np.float64)
    state0 = np.concatenate([t.h, t.hu, t.hv])
    loss, g_bed, g_src, limited = oracle.adjoint(g, dt, ticks, t.bed, t.source, state0, probes,
                                                 targets, precision64=False)
    rng = np.random.default_rng(seed + 100003 * (k + 1))
    cells = np.sort(rng.choice(t.cells, size=GRAD_CELLS, replace=False)).astype(np.int64)
    return k, dict(index=k, nx=t.nx, ny=t.ny, loss=float(loss), shortened=int(limited),
                   targets=[float(v) for v in targets], cells=[int(c) for c in cells],
                   g_bed_probes=[float(v) for v in g_bed[probes]],
                   g_src_probes=[float(v) for v in g_src[probes]],
                   g_bed_cells=[float(v) for v in g_bed[cells]],
                   g_src_cells=[float(v) for v in g_src[cells]],
                   g_bed_max=float(np.abs(g_bed).max()), g_src_max=float(np.abs(g_src).max()))


FD_TILES = (2, 10, 3, 0)  # sides 64, 128, 192, 256
FD_CELLS = 8


def _adjoint_fd_tile(k):
    import oracle
    sys.path.insert(0, os.path.dirname(HERE))
    from adjoint_cases import fd_cells
    from game_engine_gb300 import workloads as W
    t = W.tiles_256_adjoint(terrain=W.fbm_numpy, only=[k])[k]
    seed = W.SEEDS["tiles_256_adjoint"]
    ticks, dt = W.TILES_ADJOINT_TICKS, W.MAX_DT
    g = oracle.Grid(t.nx, t.ny, t.cell_m)
    tgt = oracle.RefStep(g)
    tgt.set_bed(W.perturbed_bed(t.bed, seed + k))
    tgt.set_source(t.source)
    tgt.write_state(t.h, t.hu, t.hv)
    tgt.run_steps(ticks, dt)
    probes = t.meta["probes"]
    targets = tgt.read_state_bits()[:t.cells][probes].astype(np.float64)
    state0 = np.concatenate([t.h, t.hu, t.hv])
    cells = fd_cells(dict(nx=t.nx, ny=t.ny, bed=t.bed), FD_CELLS, seed=(seed + k) & 0xFFFF,
                     eps=1e-3)
    fd_bed, fd_src = oracle.adj_fd(g, dt, ticks, t.bed, t.source, state0, probes, targets, cells,
                                   eps_bed=1e-3, rel_source=1e-3, threads=1)
    loss64 = oracle.adj_loss64(g, dt, ticks, t.bed, t.source, state0, probes, targets)
    return k, dict(index=k, nx=t.nx, ny=t.ny, cells=[int(c) for c in cells], loss_fp64=loss64,
                   fd_bed=[float(v) for v in fd_bed], fd_src=[float(v) for v in fd_src],
                   eps_bed=1e-3, rel_source=1e-3)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only",
                    default="plain_2048,tiles_4096,tiles_256_adjoint,tiles_256_adjoint_fd")
    ap.add_argument("--procs", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    import oracle
    oracle.build()
    out = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            out = json.load(f)
    out["_about"] = ("the oracle's answers on the benchmark configurations at full size "
                     "(tests/golden/make_configs.py); hashes are FNV-1a 64 over the four f32 "
                     "planes h, hu, hv, remainder (water_live.cpp:90-101)")
    only = args.only.split(",")
    ctx = mp.get_context("spawn")
    with ctx.Pool(args.procs) as pool:
        jobs = {}
        if "plain_2048" in only:
            jobs["plain_2048"] = pool.apply_async(_plain_2048)
        if "tiles_4096" in only:
            step = 64
            parts = pool.map_async(_tiles_4096_part, [(a, min(a + step, 4096))
                                                      for a in range(0, 4096, step)])
        if "tiles_256_adjoint" in only:
            adj = pool.map_async(_adjoint_tile, range(256))
        if "tiles_256_adjoint_fd" in only:
            fd = pool.map_async(_adjoint_fd_tile, FD_TILES)
        t0 = time.time()
        if "tiles_4096" in only:
            hashes = [0] * 4096
            for first, hs in parts.get():
                hashes[first:first + len(hs)] = hs
            out["tiles_4096"] = dict(count=4096, ticks=200, max_dt=0.01, hashes=hashes)
            print(f"tiles_4096 done at {time.time() - t0:.0f} s", flush=True)
        if "tiles_256_adjoint" in only:
            res = sorted(adj.get())
            out["tiles_256_adjoint"] = dict(count=256, ticks=500, every=25, max_dt=0.01,
                                            tiles=[r for _, r in res])
            print(f"tiles_256_adjoint done at {time.time() - t0:.0f} s", flush=True)
        if "tiles_256_adjoint_fd" in only:
            out["tiles_256_adjoint_fd"] = [r for _, r in fd.get()]
            print(f"tiles_256_adjoint_fd done at {time.time() - t0:.0f} s", flush=True)
        if "plain_2048" in only:
            out["plain_2048"] = jobs["plain_2048"].get()
            print(f"plain_2048 done at {time.time() - t0:.0f} s", flush=True)
    with open(OUT, "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()

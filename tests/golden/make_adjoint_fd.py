"""Writes tests/golden/adjoint_512_fd.json: central differences of the oracle's FP64 replay of the
adjoint configuration (512 x 512, 2000 fixed ticks of 0.01 s, the source on at zero, 64 probes), the check the
device's gradients are held to at full size. The replays take minutes on all host cores; the file
keeps the probes, their targets (an FP64 run on the bed plus N(0, 0.1 m)), the difference cells
(drawn away from bed ties, where the scheme has a kink) and the differences, so the test needs no
replay.

    python tests/golden/make_adjoint_fd.py [CELLS]
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from adjoint_cases import fd_cells  # noqa: E402
from game_engine_gb300 import workloads  # noqa: E402

OUT = os.path.join(HERE, "adjoint_512_fd.json")


def main():
    count = int(sys.argv[1]) if len(sys.argv) > 1 else 32
    t = workloads.adjoint_512()
    n = t.nx * t.ny
    ticks, dt = t.meta["ticks"], t.meta["max_dt"]
    g = oracle.Grid(t.nx, t.ny, t.cell_m)
    state0 = np.concatenate([t.h, t.hu, t.hv])
    probes = t.meta["probes"]
    t0 = time.time()
    fin32, limited = oracle.adj_forward(g, dt, ticks, t.bed, t.source, state0)
    print(f"FP32 forward: {limited} shortened ticks ({time.time() - t0:.0f} s)", flush=True)
    if limited:
        raise SystemExit("the configuration has shortened ticks: lower max_dt")
    bed_t = workloads.perturbed_bed(t.bed, workloads.SEEDS["adjoint_512"])
    fin_t, _ = oracle.adj_forward(g, dt, ticks, bed_t, t.source, state0, precision64=True)
    targets = fin_t[0][probes]
    loss = oracle.adj_loss64(g, dt, ticks, t.bed, t.source, state0, probes, targets)
    print(f"target run and loss {loss:.6e} ({time.time() - t0:.0f} s)", flush=True)
    c = dict(nx=t.nx, ny=t.ny, bed=t.bed)
    cells = fd_cells(c, count, seed=workloads.SEEDS["adjoint_512"] & 0xFFFF, eps=1e-3)
    fd_bed, fd_src = oracle.adj_fd(g, dt, ticks, t.bed, t.source, state0, probes, targets, cells,
                                   eps_bed=1e-3, rel_source=1e-3)
    print(f"differences at 1e-3 ({time.time() - t0:.0f} s)", flush=True)
    fd_bed_4, _ = oracle.adj_fd(g, dt, ticks, t.bed, t.source, state0, probes, targets, cells,
                                eps_bed=1e-4, with_source=False)
    print(f"differences at 1e-4 ({time.time() - t0:.0f} s)", flush=True)
    out = dict(
        config="adjoint_512", nx=t.nx, ny=t.ny, ticks=ticks, every=t.meta["every"], max_dt=dt,
        cells_total=n, loss_fp64=loss, probes=[int(p) for p in probes],
        targets=[float(v) for v in targets], fd_cells=[int(k) for k in cells],
        fd_bed=[float(v) for v in fd_bed], fd_source=[float(v) for v in fd_src],
        fd_bed_eps_small=[float(v) for v in fd_bed_4], eps_bed=1e-3, rel_source=1e-3,
        eps_bed_small=1e-4,
        fp32_final_hash=int(oracle.hash_floats(fin32.astype(np.float32).ravel())),
        command="python tests/golden/make_adjoint_fd.py " + str(count))
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()

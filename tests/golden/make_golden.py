"""Writes tests/golden/reference_fp64.json: outputs of the reference's own CPU solver
(engine::water_state::Solver, compiled from the reference's sources into oracle/_ref/libwsref.so by
oracle/build_ref.sh) on the cases below. The oracle's FP64 restatement must reproduce every hash
here byte for byte, on any host; the reference's sources are needed only to regenerate the file.

    python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

import cases  # noqa: E402
import oracle  # noqa: E402
from game_engine_gb300 import workloads  # noqa: E402


def golden_cases():
    """(name, case dict, how to run) for every golden case."""
    out = []
    for nx in (200, 400, 800):
        out.append((f"stoker_{nx}", cases.dam(nx, 0.001), dict(advance=6.0)))
        out.append((f"ritter_{nx}", cases.dam(nx, 0.0), dict(advance=6.0)))
    out.append(("exact_lake", cases.exact_lake(), dict(advance=20.0)))
    out.append(("inexact_lake", cases.inexact_lake(), dict(advance=20.0)))
    s = cases.slope(False)
    out.append(("slope_east_open_no_manning", dict(s, manning=None), dict(advance=20.0)))
    s = cases.slope(True)
    out.append(("slope_all_open_no_manning", dict(s, manning=None), dict(advance=10.0)))
    out.append(("closed_basin_300_fixed", cases.closed_basin(), dict(steps=300, max_dt=0.01)))
    t = workloads.plain_256(terrain=workloads.fbm_numpy)
    out.append(("plain_256_50_ticks", dict(nx=t.nx, ny=t.ny, cell_m=t.cell_m, bed=t.bed, h=t.h),
                dict(steps=50, max_dt=0.01)))
    return out


def run(solver_cls, name, c, how, workers=0):
    g = oracle.Grid(c["nx"], c["ny"], c["cell_m"], open_edges=c.get("open_edges", 0))
    s = solver_cls(g, workers) if workers else solver_cls(g)
    s.set_state(c["h"])
    s.set_inputs(c["bed"], c.get("manning"), c.get("source"))
    if "advance" in how:
        steps = s.advance(how["advance"])
    else:
        for _ in range(how["steps"]):
            s.step(how["max_dt"])
        steps = how["steps"]
    h, hu, hv = s.state()
    led = s.ledger()
    return dict(steps=int(steps), hash=str(s.state_hash()), volume_m3=float(s.volume()),
                source_m3=float(led["source_m3"]), open_edge_out_m3=float(led["open_edge_out_m3"]),
                roundoff_m3=float(led["roundoff_m3"]), time_s=float(led["time_s"]))


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else None
    oracle.build()
    if not oracle.build_ref(ref_root):
        raise SystemExit("the reference's sources are needed to regenerate the golden file")
    out = {"_about": "engine::water_state::Solver (the reference's own build) on these cases; "
                     "hashes are FNV-1a over h, hu, hv and the ground store as doubles "
                     "(water_state.cpp:570-578)"}
    for name, c, how in golden_cases():
        out[name] = run(oracle.RefSolver, name, c, how)
        out[name]["how"] = how
    # Thread-count invariance (water_state_tests.cpp:739-760): the same bytes on four workers.
    name, c, how = golden_cases()[-2]
    out["closed_basin_300_fixed_4_workers"] = run(oracle.RefSolver, name, c, how, workers=4)
    out["closed_basin_300_fixed_4_workers"]["how"] = how
    with open(os.path.join(HERE, "reference_fp64.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(f"wrote {len(out) - 1} golden cases")


if __name__ == "__main__":
    main()

"""Cases for the complete FP64 step (water_state::Solver with every input): the ground's store,
carried quantities, Manning's friction, sources and sinks, open edges.

Each case is a dict: the solver's configuration (`config`), its starting fields (`fields`: depth,
momenta, ground, carried), its inputs (`inputs`, the water_state::Inputs spans) and how to run it
(`run`: a list of ("step", max_dt) or ("advance", seconds)).
"""
from __future__ import annotations

import numpy as np

from cases import grid_xy, mix


def slope_full(open_edges=2, carried=2):
    """The count-of-water slope (48 x 40, device_tests.cpp:297-323) with everything on: Manning's
    n, a spring and a drain, a ground store that takes water where the bed is low, foam made by
    the dissipation and decaying, and a sediment with an outside source and an exchange with the
    bed that settles faster than the water holds it in places."""
    nx, ny = 48, 40
    cell = 0.5
    x, y = grid_xy(nx, ny)
    n = nx * ny
    bump = 0.08 * (mix(x // 3, y // 3) % 97).astype(np.float64) / 97.0
    bed = 0.6 - 0.02 * x.astype(np.float64) * cell + bump
    h = np.where(x < 12, 0.3, 0.0)
    src = np.zeros(n)
    src = np.where((x >= 20) & (x < 24) & (y >= 6) & (y < 10), 2e-3, src)
    src = np.where((x >= 30) & (x < 34) & (y >= 28) & (y < 32), -5e-3, src)
    low = x > 12
    ground_k = np.where(low, 2e-4, 0.0)
    ground_s = np.where(low, 0.05, 0.0)
    ground_cap = np.where(low, 0.02 + 0.001 * (mix(x, y) % 7), 0.0)
    cfg = dict(nx=nx, ny=ny, cell_m=cell, open_edges=open_edges,
               carried=[(30.0, 1e-4, 0.05), (0.0, 0.0, 0.0)][:carried])
    fields = dict(depth=h, momentum_x=np.zeros(n), momentum_y=np.zeros(n),
                  ground=np.where(low, 0.005, 0.0),
                  carried=np.concatenate([np.where(x < 12, 0.01, 0.0), np.where(x < 8, 0.3, 0.0)])[
                      :carried * n])
    exch = 1e-4 * ((mix(x // 2, y // 2) % 5).astype(np.float64) - 3.0)  # mostly settling
    inputs = dict(bed=bed, manning=np.full(n, 0.03), source=src, ground_k=ground_k,
                  ground_s=ground_s, ground_cap=ground_cap,
                  carried_source=[None, np.where((y > 30), 1e-4, 0.0)][:carried],
                  carried_exchange=[None, exch][:carried])
    return dict(config=cfg, fields=fields, inputs=inputs,
                run=[("step", 0.01), ("step", 0.02), ("advance", 3.0), ("step", 1.0)])


def basin_full():
    """The closed basin (96 x 64 at 0.25 m, device_tests.cpp:700-712) sloshing, no friction, with
    a foam made by the scheme's dissipation only, and a ground store everywhere."""
    nx, ny = 96, 64
    x, y = grid_xy(nx, ny)
    n = nx * ny
    bed = 0.05 * (mix(x // 4, y // 4) % 13).astype(np.float64) / 13.0
    h = np.where(x < 30, 0.8, 0.2) - bed
    cfg = dict(nx=nx, ny=ny, cell_m=0.25, open_edges=0, carried=[(0.0, 5e-5, 0.0)])
    fields = dict(depth=h, momentum_x=np.zeros(n), momentum_y=np.zeros(n), ground=np.zeros(n),
                  carried=np.zeros(n))
    inputs = dict(bed=bed, ground_k=np.full(n, 1e-5), ground_s=np.full(n, 0.1),
                  ground_cap=np.full(n, 0.05))
    return dict(config=cfg, fields=fields, inputs=inputs, run=[("advance", 2.0)])


def dam_full(nx=400):
    """Stoker's dam break (water_state_tests.cpp) with open ends and a carried dye, one row."""
    cell = 10.0 / nx
    xc = (np.arange(nx) + 0.5) * cell
    h = np.where(xc <= 5.0, 0.005, 0.001)
    cfg = dict(nx=nx, ny=1, cell_m=cell, open_edges=3, carried=[(2.0, 0.0, 0.0)])
    fields = dict(depth=h, momentum_x=np.zeros(nx), momentum_y=np.zeros(nx), ground=np.zeros(nx),
                  carried=np.where(xc <= 5.0, 0.001, 0.0))
    return dict(config=cfg, fields=fields, inputs=dict(bed=np.zeros(nx)), run=[("advance", 6.0)])


CASES = {"slope_full": slope_full, "slope_closed": lambda: slope_full(open_edges=0),
         "slope_all_open": lambda: slope_full(open_edges=15), "slope_no_carried":
         lambda: slope_full(carried=0), "basin_full": basin_full, "dam_full": dam_full}

FIELDS = ("depth", "momentum_x", "momentum_y", "ground", "carried", "speed", "bed_stress_x",
          "bed_stress_y", "dissipation")


def load(solver, case):
    for name, v in case["fields"].items():
        if name == "carried" and not case["config"]["carried"]:
            continue
        solver.set(name, v)


def run(solver, case):
    """The case's run on a solver with the oracle's interface; returns the dts and step counts."""
    out = []
    for kind, arg in case["run"]:
        if kind == "step":
            out.append(solver.step(case["inputs"], arg))
        else:
            out.append(solver.advance(case["inputs"], arg))
    return out

"""Inputs of the adjoint's tests: seeded small basins (CPU and GPU tests) and the probe-depth loss
of the adjoint configurations (a target run on the bed perturbed by Gaussian noise)."""
from __future__ import annotations

import numpy as np

import cases
import oracle


def basin(nx, ny, seed, level=3.0, edges=0, rain=1e-3, sinks=False, bump=0.4):
    """A wet basin: a smooth bed of 0-2 m with hashed roughness, the surface at `level` with a
    Gaussian bump, a uniform source (and, with `sinks`, a patch of strong sinks that dries
    cells). Returns a case dict with the state's three planes flat in `state0`."""
    x, y = cases.grid_xy(nx, ny)
    xf, yf = x.astype(np.float64), y.astype(np.float64)
    rough = (cases.mix(x + np.uint64(seed), y).astype(np.float64) % 1000) / 1000.0
    bed = 1.0 + 0.6 * np.sin(xf / 4.3) * np.cos(yf / 3.7) + 0.3 * rough
    cx, cy = 0.4 * nx, 0.55 * ny
    # a surface nowhere at rest: a lake at rest puts every face's one-sided speeds in exact ties,
    # where the scheme is not differentiable and central differences straddle the kink
    slosh = 0.05 * np.sin(xf / 2.9 + 0.3 * seed) * np.cos(yf / 3.3)
    surf = level + slosh + bump * np.exp(-((xf - cx) ** 2 + (yf - cy) ** 2) / (0.02 * nx * ny + 4.0))
    src = np.full(nx * ny, rain)
    if sinks:
        # a shoal just under the surface over strong sinks: its cells dry, the sinks run dry
        patch = (np.abs(xf - 0.7 * nx) < 3) & (np.abs(yf - 0.3 * ny) < 3)
        bed = np.where(patch, level - 0.05, bed)
        src = np.where(patch, -2.5, src)
    h = np.maximum(surf - bed, 0.0)
    return dict(nx=nx, ny=ny, cell_m=1.0, open_edges=edges, bed=bed, h=h, source=src,
                state0=np.concatenate([h, np.zeros_like(h), np.zeros_like(h)]))


def grid(c):
    return oracle.Grid(c["nx"], c["ny"], c["cell_m"], open_edges=c.get("open_edges", 0))


def probes_and_targets(c, ticks, dt, count, seed, noise=0.1):
    """`count` seeded probe cells and their targets: the FP64 fixed-step run on the bed plus
    N(0, noise) (the adjoint configurations' target run)."""
    rng = np.random.default_rng(seed)
    n = c["nx"] * c["ny"]
    probes = np.sort(rng.choice(n, size=count, replace=False)).astype(np.uint32)
    bed_t = c["bed"] + rng.normal(0.0, noise, n)
    fin, _ = oracle.adj_forward(grid(c), dt, ticks, bed_t, c.get("source"), c["state0"],
                                precision64=True)
    return probes, fin[0][probes]


def fd_cells(c, count, seed, eps):
    """`count` seeded cells for central differences of half-width `eps` on the bed, drawn among
    the cells whose bed is more than 2 eps from every neighbour's: the reconstruction takes the
    larger bed of each face (slang:274-276), so the loss has a kink where two beds tie, and a
    difference across one is not the derivative on either side."""
    nx, ny = c["nx"], c["ny"]
    z = np.asarray(c["bed"], dtype=np.float64).reshape(ny, nx)
    gap = np.full((ny, nx), np.inf)
    gap[:, 1:] = np.minimum(gap[:, 1:], np.abs(z[:, 1:] - z[:, :-1]))
    gap[:, :-1] = np.minimum(gap[:, :-1], np.abs(z[:, 1:] - z[:, :-1]))
    gap[1:, :] = np.minimum(gap[1:, :], np.abs(z[1:, :] - z[:-1, :]))
    gap[:-1, :] = np.minimum(gap[:-1, :], np.abs(z[1:, :] - z[:-1, :]))
    ok = np.nonzero(gap.ravel() > 2 * eps)[0]
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(ok, size=min(count, ok.size), replace=False)).astype(np.uint32)


def rel_err(got, want):
    """The largest error over the largest magnitude (the max-norm relative error)."""
    got, want = np.asarray(got, dtype=np.float64), np.asarray(want, dtype=np.float64)
    return float(np.max(np.abs(got - want)) / max(np.max(np.abs(want)), 1e-300))

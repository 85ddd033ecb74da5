"""Seeded synthetic inputs for the benchmark configurations (no dataset exists for this path).

Terrain is fBm: six octaves of value noise on an integer-hash lattice (the reference's `mix`,
water_live_device_tests.cpp:50-56, so the lattice is the same on every host), lacunarity 2, gain
0.5, base period side / 4, smoothstep-weighted bilinear interpolation in double, normalised to
[0, H]. Every configuration has a fixed 64-bit seed. Each workload takes its terrain generator as
`terrain`: the library's threaded `fbm` by default, or `fbm_numpy`, which gives the same doubles
without loading the library (the reference CPU arm and the fixture generators use it).

  plain_256   256 x 256, H 20 m, dry but for a centred 32 x 32 column of 2 m; 1000 ticks.
  plain_2048  2048 x 2048, H 50 m, depth U[0, 0.5] m, rain 1e-5 m a tick; 500 ticks.
  tiles_4096  4096 tiles, sides from {64, 96, 128, 192, 256, 384, 512}, each its own fBm (H 20 m)
              and a 2 m column of 32 x 32 at a seeded place; 200 ticks.
  adjoint_512 512 x 512, H 2 m, a lake: the surface at 3 m with a 0.05 m slosh and a centred
              32 x 32 column 1 m higher, the source on at zero inflow (its gradient is taken
              there); 2000 ticks, a checkpoint every 50; 64 probe cells, targets from a run on
              the bed plus N(0, 0.1 m).
  tiles_256_adjoint  256 tiles, sides from {64, 128, ..., 512}, each adjoint_512's lake on its
              own fBm; 500 ticks, a checkpoint every 25; 64 probes a tile.

The adjoint's lake is nowhere at rest: over a lake at rest every face's one-sided speeds tie
exactly, where the scheme is not differentiable. It is shallow and has no rain, because the
gradient the sweep computes is the FP32 tick's, and the check is against FP64 differences:
  - rain of 1e-5 m a tick on 20 m of water is 5.2 units in the last place of an FP32 depth, so
    each tick rounds away a fixed share of it, and the FP32 state drifts from the FP64 one by
    about 1e-3 m over 2000 ticks;
  - without rain, a 20 m lake's FP32 rounding still moves the FP32 model's gradient 1.5e-4 away
    from the FP64 model's over 2000 ticks; a 1-3 m lake's moves it 6e-5.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

SEEDS = {
    "plain_256": 0x5EED_0001_C0FF_EE01,
    "plain_2048": 0x5EED_0002_C0FF_EE02,
    "tiles_4096": 0x5EED_0003_C0FF_EE03,
    "adjoint_512": 0x5EED_0004_C0FF_EE04,
    "tiles_256_adjoint": 0x5EED_0005_C0FF_EE05,
}
ADJOINT_TICKS, ADJOINT_EVERY = 2000, 50
TILES_ADJOINT_TICKS, TILES_ADJOINT_EVERY = 500, 25
PROBES = 64
TARGET_NOISE_M = 0.1
ADJOINT_RELIEF_M, ADJOINT_LEVEL_M, ADJOINT_RISE_M = 2.0, 3.0, 1.0
MAX_DT = 0.01  # the reference's rule dt = min(stable, max_dt) with a fixed max_dt
MASK = 0xFFFFFFFF


def mix(x, y):
    x = np.asarray(x, dtype=np.uint64)
    y = np.asarray(y, dtype=np.uint64)
    h = ((x * 0x9E3779B1) & MASK) ^ ((((y + 0x7F4A7C15) & MASK) * 0x85EBCA77) & MASK)
    h ^= h >> 15
    h = (h * 0x2C1B3C6D) & MASK
    h ^= h >> 12
    return h


def _lattice(ix, iy, salt):
    return mix(ix + (salt & MASK), iy ^ ((salt >> 32) & MASK)).astype(np.float64) / 4294967296.0


def fbm(nx: int, ny: int, height: float, seed: int, octaves: int = 6) -> np.ndarray:
    """nx * ny heights in [0, height] (row-major, cell (x, y) at y * nx + x), by the library's
    threaded generator (wl_util_fbm), which gives the same doubles as fbm_numpy."""
    import ctypes as C
    from . import lib
    out = np.empty(nx * ny)
    rc = lib().wl_util_fbm(out.ctypes.data_as(C.POINTER(C.c_double)), nx, ny, float(height),
                           int(seed) & 0xFFFFFFFFFFFFFFFF, octaves)
    if rc != 0:
        raise ValueError("wl_util_fbm refused its arguments")
    return out


def fbm_numpy(nx: int, ny: int, height: float, seed: int, octaves: int = 6) -> np.ndarray:
    """The same fBm in numpy (the generator's statement; a test holds the two equal)."""
    side = max(nx, ny)
    base = max(side / 4.0, 1.0)
    ys, xs = np.meshgrid(np.arange(ny, dtype=np.float64), np.arange(nx, dtype=np.float64),
                         indexing="ij")
    total = np.zeros((ny, nx))
    amp = 1.0
    period = base
    for o in range(octaves):
        salt = (seed * (o + 1) * 0x9E3779B97F4A7C15 + o) & 0xFFFFFFFFFFFFFFFF
        fx = xs / period
        fy = ys / period
        ix = np.floor(fx)
        iy = np.floor(fy)
        tx = fx - ix
        ty = fy - iy
        sx = tx * tx * (3.0 - 2.0 * tx)
        sy = ty * ty * (3.0 - 2.0 * ty)
        ix = ix.astype(np.uint64)
        iy = iy.astype(np.uint64)
        v00 = _lattice(ix, iy, salt)
        v10 = _lattice(ix + 1, iy, salt)
        v01 = _lattice(ix, iy + 1, salt)
        v11 = _lattice(ix + 1, iy + 1, salt)
        a = v00 + (v10 - v00) * sx
        b = v01 + (v11 - v01) * sx
        total += amp * (a + (b - a) * sy)
        amp *= 0.5
        period = max(period / 2.0, 1.0)
    lo, hi = total.min(), total.max()
    span = hi - lo if hi > lo else 1.0
    return ((total - lo) / span * height).ravel()


@dataclass
class Tile:
    """One rectangle's inputs, as the API takes them (doubles, nx * ny each)."""
    nx: int
    ny: int
    bed: np.ndarray
    h: np.ndarray
    hu: np.ndarray = None
    hv: np.ndarray = None
    source: np.ndarray | None = None
    cell_m: float = 1.0
    meta: dict = field(default_factory=dict)

    def __post_init__(self):
        n = self.nx * self.ny
        if self.hu is None:
            self.hu = np.zeros(n)
        if self.hv is None:
            self.hv = np.zeros(n)

    @property
    def cells(self) -> int:
        return self.nx * self.ny


def column(nx, ny, x0, y0, side=32, depth=2.0):
    h = np.zeros((ny, nx))
    h[y0:y0 + side, x0:x0 + side] = depth
    return h.ravel()


def plain_256(terrain=fbm) -> Tile:
    n = 256
    bed = terrain(n, n, 20.0, SEEDS["plain_256"])
    h = column(n, n, n // 2 - 16, n // 2 - 16)
    return Tile(n, n, bed, h, meta=dict(ticks=1000, max_dt=MAX_DT, name="plain_256",
                                        data="synthetic: seeded 6-octave fBm terrain 0-20 m, "
                                             "dry but a centred 32 x 32 column of 2 m"))


def plain_2048(side: int = 2048, terrain=fbm) -> Tile:
    bed = terrain(side, side, 50.0, SEEDS["plain_2048"])
    rng = np.random.Generator(np.random.PCG64(SEEDS["plain_2048"] & 0xFFFFFFFF))
    h = rng.uniform(0.0, 0.5, side * side)
    rain = np.full(side * side, 1e-5 / MAX_DT)  # 1e-5 m a tick at dt = max_dt
    return Tile(side, side, bed, h, source=rain,
                meta=dict(ticks=500, max_dt=MAX_DT, name=f"plain_{side}",
                          data="synthetic: seeded 6-octave fBm terrain 0-50 m, depth U[0, 0.5] m, "
                               "rain 1e-5 m a tick"))


def full_step(side: int = 2048):
    """The complete FP64 step's workload: the throughput tile's terrain and depth with every input
    on: Manning's n 0.03, the rain, a ground store (Green-Ampt K 5e-6 m/s, suction 0.08 m,
    capacity 0.1 m), a foam made by the dissipation (decay 30 s) and a settling sediment."""
    t = plain_2048(side)
    n = t.cells
    config = dict(nx=t.nx, ny=t.ny, cell_m=t.cell_m, carried=[(30.0, 1e-4, 0.05), (0.0, 0.0, 0.0)])
    fields = dict(depth=t.h, momentum_x=t.hu, momentum_y=t.hv, ground=np.zeros(n),
                  carried=np.concatenate([np.zeros(n), 0.01 * t.h]))
    inputs = dict(bed=t.bed, manning=np.full(n, 0.03), source=t.source,
                  ground_k=np.full(n, 5e-6), ground_s=np.full(n, 0.08), ground_cap=np.full(n, 0.1),
                  carried_source=[None, None], carried_exchange=[None, np.full(n, -1e-6)])
    return t, config, fields, inputs


TILE_SIDES = (64, 96, 128, 192, 256, 384, 512)


def tile_sides(count: int, seed: int, sides=TILE_SIDES):
    rng = np.random.Generator(np.random.PCG64(seed & 0xFFFFFFFF))
    return [int(sides[k]) for k in rng.integers(0, len(sides), count)]


def tiles_4096(count: int = 4096, sides=None, seed: int | None = None, with_bed: bool = True,
               terrain=fbm, only=None):
    """The batched workload: `count` tiles of seeded sides, each its own fBm and 2 m column.
    `only`: build just these tile indices (the list holds None elsewhere; the seeded draws are the
    same)."""
    seed = SEEDS["tiles_4096"] if seed is None else seed
    sides = tile_sides(count, seed) if sides is None else sides
    keep = None if only is None else set(only)
    rng = np.random.Generator(np.random.PCG64((seed >> 32) & 0xFFFFFFFF))
    out = []
    for k, s in enumerate(sides):
        x0 = int(rng.integers(0, s - 32 + 1))
        y0 = int(rng.integers(0, s - 32 + 1))
        if keep is not None and k not in keep:
            out.append(None)
            continue
        bed = terrain(s, s, 20.0, seed + 7919 * (k + 1)) if with_bed else np.zeros(s * s)
        out.append(Tile(s, s, bed, column(s, s, x0, y0), meta=dict(index=k)))
    return out


def lake(nx, ny, bed, level=21.0, column_rise=2.0, phase=0.0):
    """Depths of a lake over `bed`: the surface at `level` with a 0.05 m slosh and a centred
    32 x 32 column `column_rise` higher."""
    ys, xs = np.meshgrid(np.arange(ny, dtype=np.float64), np.arange(nx, dtype=np.float64),
                         indexing="ij")
    slosh = 0.05 * np.sin(xs / 2.9 + phase) * np.cos(ys / 3.3)
    surf = (level + slosh).ravel() + column(nx, ny, nx // 2 - 16, ny // 2 - 16, depth=column_rise)
    return np.maximum(surf - bed, 0.0)


def probe_cells(cells: int, count: int, seed: int) -> np.ndarray:
    """`count` distinct seeded cells, sorted (a partial Fisher-Yates on the reference's hash)."""
    count = min(count, cells)
    picked = {}
    out = np.empty(count, dtype=np.uint32)
    for k in range(count):
        r = int(mix(np.uint64(k), np.uint64(seed & MASK))) % (cells - k)
        j = k + r
        out[k] = picked.get(j, j)
        picked[j] = picked.get(k, k)
    return np.sort(out)


def adjoint_512(side: int = 512, terrain=fbm) -> Tile:
    seed = SEEDS["adjoint_512"]
    bed = terrain(side, side, ADJOINT_RELIEF_M, seed)
    return Tile(side, side, bed, lake(side, side, bed, ADJOINT_LEVEL_M, ADJOINT_RISE_M),
                source=np.zeros(side * side),
                meta=dict(ticks=ADJOINT_TICKS, every=ADJOINT_EVERY, max_dt=MAX_DT,
                          name=f"adjoint_{side}",
                          probes=probe_cells(side * side, PROBES, seed)))


ADJOINT_TILE_SIDES = (64, 128, 192, 256, 320, 384, 448, 512)


def tiles_256_adjoint(count: int = 256, terrain=fbm, only=None) -> list:
    """`only`: build just these tile indices (None elsewhere), as tiles_4096."""
    seed = SEEDS["tiles_256_adjoint"]
    sides = tile_sides(count, seed, ADJOINT_TILE_SIDES)
    keep = None if only is None else set(only)
    out = []
    for k, s in enumerate(sides):
        if keep is not None and k not in keep:
            out.append(None)
            continue
        bed = terrain(s, s, ADJOINT_RELIEF_M, seed + 7919 * (k + 1))
        out.append(Tile(s, s, bed, lake(s, s, bed, ADJOINT_LEVEL_M, ADJOINT_RISE_M, phase=0.1 * k),
                        source=np.zeros(s * s),
                        meta=dict(index=k, probes=probe_cells(s * s, PROBES, seed + k))))
    return out


def perturbed_bed(bed: np.ndarray, seed: int, sigma: float = TARGET_NOISE_M) -> np.ndarray:
    """The target run's bed: `bed` plus N(0, sigma) a cell (seeded)."""
    rng = np.random.Generator(np.random.PCG64((seed >> 16) & 0xFFFFFFFF))
    return bed + rng.normal(0.0, sigma, bed.size)

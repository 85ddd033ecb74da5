"""The reference's test cases as inputs, restated from its tests (systems/water_live/tests/
water_live_device_tests.cpp, domain/water_state/tests/water_state_tests.cpp) and the seeded
synthetic workloads of the benchmark configurations. Every input is built from integer hashing and
plain double arithmetic, so it is the same on every host (no libm)."""
from __future__ import annotations

import numpy as np

MASK = 0xFFFFFFFF


def mix(x, y):
    """The reference's integer hash (water_live_device_tests.cpp:50-56), vectorised over uint32."""
    x = np.asarray(x, dtype=np.uint64)
    y = np.asarray(y, dtype=np.uint64)
    h = ((x * 0x9E3779B1) & MASK) ^ (((y + 0x7F4A7C15) & MASK) * 0x85EBCA77 & MASK)
    h &= MASK
    h ^= h >> 15
    h = (h * 0x2C1B3C6D) & MASK
    h ^= h >> 12
    return h.astype(np.uint64)


def grid_xy(nx, ny):
    y, x = np.meshgrid(np.arange(ny, dtype=np.uint64), np.arange(nx, dtype=np.uint64),
                       indexing="ij")
    return x.ravel(), y.ravel()


def exact_lake():
    """64 x 48, 0.5 m cells, binary-fraction bed with islands (device_tests.cpp:200-219)."""
    nx, ny = 64, 48
    x, y = grid_xy(nx, ny)
    z = ((x * 7 + y * 13) % 17).astype(np.float64) / 64.0
    island = (((x // 8 + y // 8) % 3) == 0) & ((x % 8) > 1) & ((y % 8) > 2)
    z = np.where(island, 1.0 + (mix(x, y) % 16).astype(np.float64) / 64.0, z)
    h = np.maximum(1.0 - z, 0.0)
    return dict(nx=nx, ny=ny, cell_m=0.5, bed=z, h=h)


def inexact_lake():
    """device_tests.cpp:221-240."""
    nx, ny = 64, 48
    x, y = grid_xy(nx, ny)
    z = 0.731 * (mix(x, y) % 1001).astype(np.float64) / 1001.0
    island = (((x // 8 + y // 8) % 3) == 0) & ((x % 8) > 1) & ((y % 8) > 2)
    z = np.where(island, 0.9 + 0.37 * (mix(y, x) % 101).astype(np.float64) / 101.0, z)
    h = np.maximum(0.9 - z, 0.0)
    return dict(nx=nx, ny=ny, cell_m=0.5, bed=z, h=h)


def dam(nx, hr):
    """Stoker (hr > 0) and Ritter (hr = 0) on 10 m (device_tests.cpp:102-113)."""
    cell = 10.0 / nx
    xc = (np.arange(nx) + 0.5) * cell
    h = np.where(xc <= 5.0, 0.005, hr)
    return dict(nx=nx, ny=1, cell_m=cell, bed=np.zeros(nx), h=h.astype(np.float64))


def slope(all_open=False):
    """The count of water: 48 x 40 slope, n = 0.03, a spring and a drain (device_tests.cpp:297-323)."""
    nx, ny = 48, 40
    cell = 0.5
    x, y = grid_xy(nx, ny)
    bump = 0.08 * (mix(x // 3, y // 3) % 97).astype(np.float64) / 97.0
    bed = 0.6 - 0.02 * x.astype(np.float64) * cell + bump
    h = np.where(x < 12, 0.3, 0.0)
    src = np.zeros(nx * ny)
    src = np.where((x >= 20) & (x < 24) & (y >= 6) & (y < 10), 2e-3, src)
    src = np.where((x >= 30) & (x < 34) & (y >= 28) & (y < 32), -5e-3, src)
    open_edges = 15 if all_open else 2
    return dict(nx=nx, ny=ny, cell_m=cell, bed=bed, h=h, manning=np.full(nx * ny, 0.03),
                source=src, open_edges=open_edges)


def closed_basin():
    """96 x 64 at 0.25 m, a dam break sloshing (device_tests.cpp:700-712)."""
    nx, ny = 96, 64
    x, y = grid_xy(nx, ny)
    bed = 0.05 * (mix(x // 4, y // 4) % 13).astype(np.float64) / 13.0
    h = np.where(x < 30, 0.8, 0.2) - bed
    return dict(nx=nx, ny=ny, cell_m=0.25, bed=bed, h=h)

"""The batched form over the C ABI (include/wlcuda.h, wl_batch_*): many tiles of uneven sizes,
one persistent CUDA-graph-captured launch per tick, and the per-tile-launch form beside it.

Each tile steps exactly as a DeviceStep of its size would (the same bytes); whole-batch arrays hold
every tile's cells tile after tile.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi, lib
from .water_live import OPS_FIXED, OPS_NATIVE, STATE_PLANES

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)


class BatchError(RuntimeError):
    pass


class Batch:
    def __init__(self, sides, cell_m=1.0, gravity=9.81, cfl=0.45, dry_depth_m=1e-9,
                 open_edges=None, fixed=False, device=0):
        """`sides`: a list of (nx, ny); `open_edges`: per tile bits (1 W, 2 E, 4 S, 8 N)."""
        self._buf = C.create_string_buffer(512)
        n = len(sides)
        tiles = (_abi.Tile * n)()
        for k, (nx, ny) in enumerate(sides):
            e = 0 if open_edges is None else int(open_edges[k])
            tiles[k] = _abi.Tile(int(nx), int(ny), e & 1, (e >> 1) & 1, (e >> 2) & 1, (e >> 3) & 1)
        cfg = _abi.Config(0, 0, cell_m, gravity, cfl, dry_depth_m, 0, 0, 0, 0, device)
        opts = _abi.Options(OPS_FIXED if fixed else OPS_NATIVE, 0)
        h = C.c_void_p()
        self._h = None
        self._check(lib().wl_batch_create(C.byref(cfg), C.byref(opts), tiles, n, C.byref(h),
                                          self._buf, len(self._buf)))
        self._h = h
        self.sides = [(int(a), int(b)) for a, b in sides]
        self.first = np.array([lib().wl_batch_tile_first(self._h, k) for k in range(n)],
                              dtype=np.int64)
        self.cells = int(lib().wl_batch_cell_count(self._h))

    def _check(self, rc):
        if rc != 0:
            raise BatchError(self._buf.value.decode() or f"wlcuda error {rc}")

    def close(self):
        if self._h is not None:
            lib().wl_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def tile_count(self):
        return len(self.sides)

    def tile_slice(self, k):
        nx, ny = self.sides[k]
        return slice(int(self.first[k]), int(self.first[k]) + nx * ny)

    def _arr(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size != self.cells:
            raise BatchError("water_live: arrays that do not fit the tiles")
        return a

    def write_state(self, h, hu=None, hv=None):
        h = self._arr(h)
        hu = self._arr(np.zeros(self.cells) if hu is None else hu)
        hv = self._arr(np.zeros(self.cells) if hv is None else hv)
        self._check(lib().wl_batch_write_state(self._h, h.ctypes.data_as(_dp),
                                               hu.ctypes.data_as(_dp), hv.ctypes.data_as(_dp),
                                               self.cells, self._buf, len(self._buf)))

    def write_tile_state(self, tile, h, hu=None, hv=None):
        """One tile's state between ticks (its ledger emptied, its records primed); the other
        tiles are untouched: the tile-start upload of a tile that wakes."""
        nx, ny = self.sides[tile]
        n = nx * ny
        h = np.ascontiguousarray(h, dtype=np.float64)
        hu = np.ascontiguousarray(np.zeros(n) if hu is None else hu, dtype=np.float64)
        hv = np.ascontiguousarray(np.zeros(n) if hv is None else hv, dtype=np.float64)
        if not (h.size == hu.size == hv.size):
            raise BatchError("water_live: spans of different sizes")
        self._check(lib().wl_batch_write_tile_state(self._h, int(tile), h.ctypes.data_as(_dp),
                                                    hu.ctypes.data_as(_dp),
                                                    hv.ctypes.data_as(_dp), h.size, self._buf,
                                                    len(self._buf)))

    def settled(self, h, hu, hv, depth_bound_m, momentum_bound_m2_s):
        """The settled check of every tile against a steady state (whole-batch arrays, tile after
        tile): (settled bools, depth deviations, momentum deviations), one each a tile."""
        h, hu, hv = self._arr(h), self._arr(hu), self._arr(hv)
        n = self.tile_count
        ok8 = np.zeros(n, dtype=np.uint8)
        dd = np.zeros(n, dtype=np.float32)
        dq = np.zeros(n, dtype=np.float32)
        self._check(lib().wl_batch_settled(self._h, h.ctypes.data_as(_dp), hu.ctypes.data_as(_dp),
                                           hv.ctypes.data_as(_dp), self.cells,
                                           float(depth_bound_m), float(momentum_bound_m2_s),
                                           ok8.ctypes.data_as(C.POINTER(C.c_uint8)),
                                           dd.ctypes.data_as(_fp), dq.ctypes.data_as(_fp), n,
                                           self._buf, len(self._buf)))
        return ok8.astype(bool), dd, dq

    def set_bed(self, bed, datum=0.0):
        b = self._arr(bed)
        self._check(lib().wl_batch_set_bed(self._h, b.ctypes.data_as(_dp), self.cells,
                                           float(datum), self._buf, len(self._buf)))

    def set_manning(self, m):
        if m is None:
            self._check(lib().wl_batch_set_manning(self._h, None, 0, self._buf, len(self._buf)))
            return
        m = self._arr(m)
        self._check(lib().wl_batch_set_manning(self._h, m.ctypes.data_as(_dp), self.cells,
                                               self._buf, len(self._buf)))

    def set_source(self, s, every=1, compensate=False):
        if s is None:
            self._check(lib().wl_batch_set_source(self._h, None, 0, int(every), int(compensate),
                                                  self._buf, len(self._buf)))
            return
        s = self._arr(s)
        self._check(lib().wl_batch_set_source(self._h, s.ctypes.data_as(_dp), self.cells,
                                              int(every), int(compensate), self._buf,
                                              len(self._buf)))

    def run_ticks(self, count, max_dt, graph=True):
        self._check(lib().wl_batch_run_ticks(self._h, int(count), float(max_dt), int(graph),
                                             self._buf, len(self._buf)))

    def enqueue_ticks(self, stream, count, max_dt):
        self._check(lib().wl_batch_enqueue_ticks(self._h, stream, int(count), float(max_dt)))

    def run_tile_ticks(self, count, max_dt, graph=True, streams=1):
        self._check(lib().wl_batch_run_tile_ticks(self._h, int(count), float(max_dt), int(graph),
                                                  int(streams), self._buf, len(self._buf)))

    def read_tile_bits(self, k):
        nx, ny = self.sides[k]
        out = np.empty(STATE_PLANES * nx * ny, dtype=np.float32)
        self._check(lib().wl_batch_read_tile_bits(self._h, int(k), out.ctypes.data_as(_fp),
                                                  out.size, self._buf, len(self._buf)))
        return out

    def tile_hash(self, k):
        h = int(lib().wl_batch_tile_hash(self._h, int(k), self._buf, len(self._buf)))
        if h == 0:
            raise BatchError(self._buf.value.decode())
        return h

    def tile_hashes(self):
        out = np.zeros(self.tile_count, dtype=np.uint64)
        self._check(lib().wl_batch_tile_hashes(self._h, out.ctypes.data_as(C.POINTER(C.c_uint64)),
                                               self.tile_count, self._buf, len(self._buf)))
        return out

    def ledgers(self):
        arr = (_abi.Ledger * self.tile_count)()
        self._check(lib().wl_batch_read_ledgers(self._h, arr, self.tile_count, self._buf,
                                                len(self._buf)))
        return [dict(source_m3=l.source_m3, open_edge_out_m3=l.open_edge_out_m3,
                     roundoff_m3=l.roundoff_m3, time_s=l.time_s, remaining_s=l.remaining_s,
                     steps=int(l.steps)) for l in arr]

    def autotune(self, max_dt, trial_ticks=4):
        t = _abi.Tuning()
        self._check(lib().wl_batch_autotune(self._h, float(max_dt), int(trial_ticks), C.byref(t),
                                            self._buf, len(self._buf)))
        return dict(block_rows=t.block_rows, order=t.order, us_per_tick=t.us_per_tick,
                    zero_apart=t.zero_apart, stage=t.stage)

    def set_tuning(self, block_rows, order, zero_apart=0, stage=0):
        t = _abi.Tuning(int(block_rows), int(order), 0.0, int(zero_apart), int(stage))
        self._check(lib().wl_batch_set_tuning(self._h, C.byref(t), self._buf, len(self._buf)))

    def tuning(self):
        t = _abi.Tuning()
        self._check(lib().wl_batch_get_tuning(self._h, C.byref(t)))
        return dict(block_rows=t.block_rows, order=t.order, us_per_tick=t.us_per_tick,
                    zero_apart=t.zero_apart, stage=t.stage)

    def stream(self):
        return lib().wl_batch_stream(self._h)

    def staged_tiles(self):
        """Tiles whose blocks the batch's launches take by tensor copies under its tuning."""
        return int(lib().wl_batch_staged_tiles(self._h))


def concat(tiles, field):
    """One field of a list of workloads.Tile, tile after tile."""
    return np.concatenate([getattr(t, field) for t in tiles])

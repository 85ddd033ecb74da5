"""The adjoint over the C ABI (include/wlcuda.h, wl_adjoint_*): gradients of a probe-depth loss
with respect to the bed and the per-cell source, by a checkpointed reverse sweep on the device.

The loss is L = sum over probe cells p of (h_T(p) - target_p)^2 after T ticks of fixed length
from the owner's current state. Over a DeviceStep there is one loss; over a Batch, one a tile.
The reference has no adjoint; the sweep's forward ticks are the plain tick to the bit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_u32p = C.POINTER(C.c_uint32)


class AdjointError(RuntimeError):
    pass


class Adjoint:
    def __init__(self, owner, ticks: int, every: int, probes, targets):
        """`owner`: a DeviceStep or a Batch (which must outlive the sweep). Over a step, `probes`
        and `targets` are arrays of cells (y * nx + x) and depths; over a batch, lists with one
        such array a tile (tile-local cells)."""
        from .batch import Batch

        self._buf = C.create_string_buffer(512)
        self._h = None
        self.owner = owner
        self.ticks = int(ticks)
        self.every = int(every)
        h = C.c_void_p()
        if isinstance(owner, Batch):
            self.tiles = len(owner.sides)
            counts = [len(p) for p in probes]
            if len(counts) != self.tiles or len(targets) != self.tiles:
                raise AdjointError("one probe array and one target array a tile")
            first = np.zeros(self.tiles + 1, dtype=np.uint32)
            first[1:] = np.cumsum(counts)
            pr = np.ascontiguousarray(np.concatenate([np.asarray(p, dtype=np.uint32)
                                                      for p in probes]) if self.tiles else [],
                                      dtype=np.uint32)
            tg = np.ascontiguousarray(np.concatenate([np.asarray(t, dtype=np.float64)
                                                      for t in targets]), dtype=np.float64)
            self._keep = (first, pr, tg)
            rc = lib().wl_batch_adjoint_create(owner._h, self.ticks, self.every,
                                               first.ctypes.data_as(_u32p),
                                               pr.ctypes.data_as(_u32p), tg.ctypes.data_as(_dp),
                                               C.byref(h), self._buf, len(self._buf))
            self.cells = owner.cells
        else:
            self.tiles = 1
            pr = np.ascontiguousarray(probes, dtype=np.uint32)
            tg = np.ascontiguousarray(targets, dtype=np.float64)
            if pr.size != tg.size:
                raise AdjointError("one target a probe")
            self._keep = (pr, tg)
            rc = lib().wl_adjoint_create(owner.handle, self.ticks, self.every, pr.size,
                                         pr.ctypes.data_as(_u32p), tg.ctypes.data_as(_dp),
                                         C.byref(h), self._buf, len(self._buf))
            self.cells = owner.cell_count()
        self._check(rc)
        self._h = h

    def _check(self, rc):
        if rc != 0:
            raise AdjointError(self._buf.value.decode() or f"wlcuda error {rc}")

    def close(self):
        if self._h is not None:
            lib().wl_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, max_dt: float, graph: bool = True) -> None:
        self._check(lib().wl_adjoint_run(self._h, float(max_dt), int(graph), self._buf,
                                         len(self._buf)))

    def enqueue(self, max_dt: float) -> None:
        rc = lib().wl_adjoint_enqueue(self._h, float(max_dt))
        if rc != 0:
            raise AdjointError(f"wl_adjoint_enqueue: error {rc}")

    def read(self):
        """(loss a tile, dL/d(bed) a cell, dL/d(source) a cell, shortened ticks a tile)."""
        loss = np.zeros(self.tiles)
        g_bed = np.zeros(self.cells)
        g_src = np.zeros(self.cells)
        limited = np.zeros(self.tiles, dtype=np.uint32)
        self._check(lib().wl_adjoint_read(self._h, loss.ctypes.data_as(_dp),
                                          g_bed.ctypes.data_as(_dp), g_src.ctypes.data_as(_dp),
                                          limited.ctypes.data_as(_u32p), self._buf,
                                          len(self._buf)))
        return loss, g_bed, g_src, limited

    def read_final(self):
        """The state of tick T: three planes (h, hu, hv) a tile, tile after tile (flat)."""
        out = np.zeros(3 * self.cells, dtype=np.float32)
        self._check(lib().wl_adjoint_read_final(self._h, out.ctypes.data_as(_fp), self._buf,
                                                len(self._buf)))
        return out

    def read_state_gradient(self):
        """dL/d(starting state): three planes (dL/dh, dL/dhu, dL/dhv) a tile, tile after tile
        (flat, FP32)."""
        out = np.zeros(3 * self.cells, dtype=np.float32)
        self._check(lib().wl_adjoint_read_state_gradient(self._h, out.ctypes.data_as(_fp),
                                                         self._buf, len(self._buf)))
        return out

    def launches(self) -> int:
        return int(lib().wl_adjoint_launches(self._h))

    def device_bytes(self) -> int:
        return int(lib().wl_adjoint_device_bytes(self._h))

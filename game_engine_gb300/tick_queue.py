"""The tick queue over the C ABI (include/wlcuda.h, "the tick queue").

The design is the reference's (docs/subsystems/water_live.md:76-94, ADR-0081), which the reference
has not built: ticks of the world's clock, each a length and the events that take effect at its
start, queued on the device and stepped by sub-step slots. Calls that move data return
``True``/``False`` and leave the message in :attr:`TickQueue.error`, as ``DeviceStep`` does.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi, lib

EVENT_BED, EVENT_SOURCE, EVENT_MANNING, EVENT_STATE = 0, 1, 2, 3
ERR_REFUSED = 5
MAX_RECORDS = 64

_fp = C.POINTER(C.c_float)


@dataclass
class Event:
    """A rectangle of one plane (EVENT_*) of one tile replaced by ``values`` (h rows of w, row by
    row); tile 0 for a step's queue. An EVENT_STATE's values are (3, h, w): depth, then the two
    momenta (a waking tile's starting state)."""
    kind: int
    x0: int
    y0: int
    values: np.ndarray  # shape (h, w), or (3, h, w) for EVENT_STATE
    tile: int = 0


class TickQueue:
    """The queue of ticks over one ``water_live.DeviceStep`` or one ``batch.Batch`` (the domain's
    tiles take every tick together, each by its own sub-steps)."""

    def __init__(self, owner, records: int = MAX_RECORDS, arena_values: int = 1 << 16,
                 max_events: int = 256):
        from .batch import Batch
        self.error = ""
        self.last_code = 0
        self._buf = C.create_string_buffer(512)
        self._h = None
        self._owner = owner
        h = C.c_void_p()
        create = lib().wl_batch_queue_create if isinstance(owner, Batch) else lib().wl_queue_create
        rc = create(owner.handle, int(records), int(arena_values), int(max_events), C.byref(h),
                    self._buf, len(self._buf))
        if rc != 0:
            raise RuntimeError(self._buf.value.decode())
        self._h = h

    def close(self) -> None:
        if self._h is not None:
            lib().wl_queue_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc: int) -> bool:
        self.last_code = rc
        if rc != 0:
            self.error = self._buf.value.decode()
            return False
        return True

    def push(self, tick: int, length_s: float, events=()) -> bool:
        """Queues one tick; False with ``last_code`` ERR_REFUSED when the queue has no room yet."""
        evs = (_abi.Event * max(len(events), 1))()
        vals = []
        for k, e in enumerate(events):
            v = np.ascontiguousarray(e.values, dtype=np.float32)
            h, w = v.shape[-2:]
            evs[k] = _abi.Event(int(e.kind), int(e.x0), int(e.y0), int(w), int(h), int(e.tile))
            vals.append(v.ravel())
        flat = np.concatenate(vals) if vals else np.zeros(1, np.float32)
        n_values = int(sum(v.size for v in vals))
        return self._ok(lib().wl_queue_push(self._h, int(tick) & 0xFFFFFFFF, float(length_s), evs,
                                            len(events), flat.ctypes.data_as(_fp), n_values,
                                            self._buf, len(self._buf)))

    def enqueue_slots(self, stream, slots: int) -> bool:
        """``slots`` slots on a CUDA stream (an int handle, or None for the step's own); no wait."""
        rc = lib().wl_queue_enqueue_slots(self._h, stream, int(slots))
        if rc != 0:
            self.error = f"water_live: enqueue of the slots failed ({rc})"
            self.last_code = rc
            return False
        return True

    def set_limits(self, lag_limit_ticks: int = 0, max_slots: int = 0) -> bool:
        """The lag control (water_live.md:90-92): past ``lag_limit_ticks`` ticks pushed and not
        landed the domain freezes and drops ticks until the queue drains; ``max_slots`` caps the
        slots one call enqueues. 0 turns either off."""
        return self._ok(lib().wl_queue_set_limits(self._h, int(lag_limit_ticks), int(max_slots),
                                                  self._buf, len(self._buf)))

    def run_slots(self, slots: int) -> bool:
        return self._ok(lib().wl_queue_run_slots(self._h, int(slots), self._buf, len(self._buf)))

    def status(self):
        s = _abi.QueueStatus()
        if not self._ok(lib().wl_queue_status_read(self._h, C.byref(s), self._buf,
                                                   len(self._buf))):
            return None
        return dict(pushed=s.pushed, begun=s.begun, landed=s.landed, active=s.active,
                    substeps=s.substeps, dropped=s.dropped, frozen=s.frozen, freezes=s.freezes)

    def landed(self, first: int, count: int):
        """The read-back records of landings first .. first + count - 1, as dicts."""
        out = (_abi.Landed * max(count, 1))()
        if not self._ok(lib().wl_queue_read_landed(self._h, int(first), int(count), out,
                                                   self._buf, len(self._buf))):
            return None
        return [dict(tick=r.tick, substeps=r.substeps, shortest_s=r.shortest_s,
                     longest_s=r.longest_s, time_hi=r.time_hi, time_lo=r.time_lo, steps=r.steps,
                     events=r.events, dropped=r.dropped, dropped_total=r.dropped_total,
                     lag=r.lag, frozen=r.frozen) for r in out[:count]]

    @staticmethod
    def launches_per_slot() -> int:
        return int(lib().wl_queue_launches_per_slot())

    def device_bytes(self) -> int:
        return int(lib().wl_queue_device_bytes(self._h)) if self._h is not None else 0

"""water_live::DeviceStep's interface over the C ABI (include/wlcuda.h).

The method set and the error behaviour are the reference's
(systems/water_live/include/systems/water_live/water_live.h:158-256): calls that move data return
``True``/``False`` and leave the message in :attr:`DeviceStep.error`; ``advance`` and
``state_hash`` return 0 on an error; a step that was never created refuses every call.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi, lib

OPS_NATIVE = 0
OPS_FIXED = 1
STATE_PLANES = 4
GROUP_SIDE = 16
FLAG_WEST_OPEN, FLAG_EAST_OPEN, FLAG_SOUTH_OPEN, FLAG_NORTH_OPEN = 1, 2, 4, 8
FLAG_MANNING, FLAG_SOURCE, FLAG_COMPENSATE, FLAG_STORED_FACES = 16, 32, 64, 128

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)


@dataclass
class Config:
    """water_state::Config (water_state.h:83-99): the fields the step reads."""
    nx: int
    ny: int
    cell_m: float = 1.0
    gravity: float = 9.81
    cfl: float = 0.45
    dry_depth_m: float = 1e-9
    west_open: bool = False
    east_open: bool = False
    south_open: bool = False
    north_open: bool = False
    device: int = 0

    @property
    def open_edges(self) -> int:
        return (int(self.west_open) | int(self.east_open) << 1 | int(self.south_open) << 2
                | int(self.north_open) << 3)

    def to_c(self) -> _abi.Config:
        return _abi.Config(self.nx, self.ny, self.cell_m, self.gravity, self.cfl,
                           self.dry_depth_m, int(self.west_open), int(self.east_open),
                           int(self.south_open), int(self.north_open), self.device)


@dataclass
class StepOptions:
    """water_live::StepOptions (water_live.h:105-110)."""
    ops: int = OPS_NATIVE
    stored_faces: bool = False


def _f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a


def hash_floats(values) -> int:
    """water_live::hash_floats (water_live.cpp:90-101): FNV-1a over float bytes."""
    v = np.ascontiguousarray(values, dtype=np.float32)
    return int(lib().wl_hash_floats(v.ctypes.data_as(_fp), v.size))


class DeviceStep:
    """One rectangle of water on a GB300: the reference's DeviceStep (water_live.h:158-256)."""

    def __init__(self):
        self._h = None
        self.error = ""
        self._buf = C.create_string_buffer(512)
        self._config = None
        self._options = StepOptions()

    # -- lifecycle ---------------------------------------------------------------------------
    def create(self, config: Config, options: StepOptions | None = None) -> bool:
        self.destroy()
        options = options or StepOptions()
        handle = C.c_void_p()
        rc = lib().wl_create(C.byref(config.to_c()),
                             C.byref(_abi.Options(options.ops, int(options.stored_faces))),
                             C.byref(handle), self._buf, len(self._buf))
        if rc != 0:
            self.error = self._buf.value.decode()
            return False
        self._h = handle
        self._config = config
        self._options = options
        return True

    def destroy(self) -> None:
        if self._h is not None:
            lib().wl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def valid(self) -> bool:
        return self._h is not None and bool(lib().wl_valid(self._h))

    @property
    def handle(self):
        return self._h

    def config(self) -> Config:
        return self._config

    def options(self) -> StepOptions:
        return self._options

    def cell_count(self) -> int:
        return int(lib().wl_cell_count(self._h)) if self._h is not None else 0

    def group_count(self) -> int:
        return int(lib().wl_group_count(self._h)) if self._h is not None else 0

    def _ok(self, rc: int) -> bool:
        if rc != 0:
            self.error = self._buf.value.decode()
            self.last_code = rc
            return False
        return True

    # -- data ----------------------------------------------------------------------------------
    def write_state(self, depth, momentum_x, momentum_y) -> bool:
        h, hu, hv = _f64(depth), _f64(momentum_x), _f64(momentum_y)
        if not (h.size == hu.size == hv.size):
            self.error = "water_live: a state that does not fit the grid"
            return False
        return self._ok(lib().wl_write_state(self._h, h.ctypes.data_as(_dp), hu.ctypes.data_as(_dp),
                                             hv.ctypes.data_as(_dp), h.size, self._buf,
                                             len(self._buf)))

    def read_state(self):
        n = self.cell_count()
        h, hu, hv = np.empty(n), np.empty(n), np.empty(n)
        ok = self._ok(lib().wl_read_state(self._h, h.ctypes.data_as(_dp), hu.ctypes.data_as(_dp),
                                          hv.ctypes.data_as(_dp), n, self._buf, len(self._buf)))
        return (h, hu, hv) if ok else None

    def read_state_bits(self):
        n = STATE_PLANES * self.cell_count()
        out = np.empty(n, dtype=np.float32)
        ok = self._ok(lib().wl_read_state_bits(self._h, out.ctypes.data_as(_fp), n, self._buf,
                                               len(self._buf)))
        return out if ok else None

    def read_ledger(self):
        out = _abi.Ledger()
        if not self._ok(lib().wl_read_ledger(self._h, C.byref(out), self._buf, len(self._buf))):
            return None
        return dict(source_m3=out.source_m3, open_edge_out_m3=out.open_edge_out_m3,
                    roundoff_m3=out.roundoff_m3, time_s=out.time_s, remaining_s=out.remaining_s,
                    steps=int(out.steps))

    def settled(self, h, hu, hv, depth_bound_m: float, momentum_bound_m2_s: float):
        """The settled check against a steady state (ADR-0080 decision 4): (settled, largest depth
        deviation, largest momentum deviation), or None on an error."""
        h, hu, hv = _f64(h), _f64(hu), _f64(hv)
        ok8 = C.c_uint8(0)
        dd, dq = C.c_float(0.0), C.c_float(0.0)
        if not self._ok(lib().wl_settled(self._h, h.ctypes.data_as(_dp), hu.ctypes.data_as(_dp),
                                         hv.ctypes.data_as(_dp), h.size, float(depth_bound_m),
                                         float(momentum_bound_m2_s), C.byref(ok8), C.byref(dd),
                                         C.byref(dq), self._buf, len(self._buf))):
            return None
        return bool(ok8.value), float(dd.value), float(dq.value)

    def set_bed(self, bed_m, datum_m: float = 0.0) -> bool:
        b = _f64(bed_m)
        return self._ok(lib().wl_set_bed(self._h, b.ctypes.data_as(_dp), b.size, float(datum_m),
                                         self._buf, len(self._buf)))

    def set_manning(self, manning) -> bool:
        m = _f64(manning if manning is not None else [])
        return self._ok(lib().wl_set_manning(self._h, m.ctypes.data_as(_dp), m.size, self._buf,
                                             len(self._buf)))

    def set_source(self, source_m_per_s, every: int = 1, compensate: bool = False) -> bool:
        s = _f64(source_m_per_s if source_m_per_s is not None else [])
        return self._ok(lib().wl_set_source(self._h, s.ctypes.data_as(_dp), s.size, int(every),
                                            int(bool(compensate)), self._buf, len(self._buf)))

    # -- steps ---------------------------------------------------------------------------------
    def record(self, stream, count: int, max_dt: float) -> bool:
        """DeviceStep::record onto a CUDA stream (an int handle or None for the step's own)."""
        if self._h is None:
            self.error = "water_live: no device"
            return False
        rc = lib().wl_enqueue_steps(self._h, stream, int(count), float(max_dt))
        if rc != 0:
            self.error = f"water_live: enqueue failed ({rc})"
            return False
        return True

    def tick_launches(self) -> int:
        """Tick kernel launches enqueued since create (a diagnosis counter): a small tile steps a
        call's ticks in one resident launch, a larger one a launch a tick."""
        return int(lib().wl_tick_launches(self._h)) if self._h is not None else 0

    def staged_tiles(self) -> int:
        """1 where the step's three-phase blocks take their cells and halo by tensor copies (a
        width that is a multiple of 4, and more blocks than the launch's 256-thread CTAs, or
        WLCUDA_STAGE=1 at create), else 0."""
        return int(lib().wl_staged_tiles(self._h)) if self._h is not None else 0

    def run_steps(self, count: int, max_dt: float) -> bool:
        return self._ok(lib().wl_run_steps(self._h, int(count), float(max_dt), self._buf,
                                           len(self._buf)))

    def advance(self, duration_s: float) -> int:
        steps = int(lib().wl_advance(self._h, float(duration_s), self._buf, len(self._buf)))
        if steps == 0:
            self.error = self._buf.value.decode()
        return steps

    def state_hash(self) -> int:
        h = int(lib().wl_state_hash(self._h, self._buf, len(self._buf)))
        if h == 0:
            self.error = self._buf.value.decode()
        return h

    # -- diagnosis -----------------------------------------------------------------------------
    def read_partials_bits(self):
        g = self.group_count()
        arr = (_abi.Partial * max(g, 1))()
        if not self._ok(lib().wl_read_partials_bits(self._h, arr, g, self._buf, len(self._buf))):
            return None
        return np.frombuffer(bytes(arr), dtype=np.float32).reshape(-1, 8)[:g].copy()

    def read_ledger_bits(self):
        out = _abi.LedgerBits()
        if not self._ok(lib().wl_read_ledger_bits(self._h, C.byref(out), self._buf,
                                                  len(self._buf))):
            return None
        return np.frombuffer(bytes(out), dtype=np.uint32).copy()

    def run_length_pass(self, max_dt: float) -> bool:
        return self._ok(lib().wl_run_length_pass(self._h, float(max_dt), self._buf,
                                                 len(self._buf)))

    def stream(self):
        return lib().wl_step_stream(self._h) if self._h is not None else None

    def device_planes(self):
        """(planes, bed) device pointers of the current copy (ints)."""
        p, b = _fp(), _fp()
        if not self._ok(lib().wl_device_planes(self._h, C.byref(p), C.byref(b), self._buf,
                                               len(self._buf))):
            return None
        return C.cast(p, C.c_void_p).value, C.cast(b, C.c_void_p).value

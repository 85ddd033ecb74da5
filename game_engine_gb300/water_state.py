"""engine::water_state::Solver on the device, over the C ABI (include/wlcuda.h, "the complete FP64
step").

The reference's complete FP64 step (domain/water_state/include/domain/water_state/water_state.h:
161-266): the state's fields (depth, momenta, the ground's store, carried quantities), the last
step's outputs (speed, bed stress, dissipation), `step`, `advance`, `stable_step`, the ledger,
the volumes and `state_hash`, with the bytes of the reference's CPU step. Inputs are a dict of the
reference's Inputs spans (bed, manning, source, ground_k, ground_s, ground_cap, carried_source,
carried_exchange); `step` and `advance` upload what changed and keep it on the device.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi, lib

FIELDS = dict(depth=0, momentum_x=1, momentum_y=2, ground=3, carried=4, speed=5,
              bed_stress_x=6, bed_stress_y=7, dissipation=8)
INPUTS = dict(bed=0, manning=1, source=2, ground_k=3, ground_s=4, ground_cap=5)
CARRIED_SOURCE, CARRIED_EXCHANGE = 6, 10
LEDGER_KEYS = ("source_m3", "open_edge_out_m3", "ground_m3", "roundoff_m3", "scheme_loss_j",
               "friction_work_j", "time_s", "steps")
CARRIED_LEDGER_KEYS = ("source", "from_dissipation", "exchange", "decayed", "open_edge_out")

_dp = C.POINTER(C.c_double)


@dataclass
class Config:
    """water_state::Config (water_state.h:83-99). `carried` lists each quantity's
    (decay_s, per_joule, min_speed_m_per_s)."""
    nx: int
    ny: int
    cell_m: float = 1.0
    gravity: float = 9.81
    cfl: float = 0.45
    dry_depth_m: float = 1e-9
    water_density: float = 1000.0
    carried: list = field(default_factory=list)
    west_open: bool = False
    east_open: bool = False
    south_open: bool = False
    north_open: bool = False
    device: int = 0

    def to_c(self) -> _abi.WsConfig:
        c = _abi.WsConfig()
        c.nx, c.ny = self.nx, self.ny
        c.cell_m, c.gravity, c.cfl = self.cell_m, self.gravity, self.cfl
        c.dry_depth_m, c.water_density = self.dry_depth_m, self.water_density
        c.carried = len(self.carried)
        for k, (decay, per_joule, min_speed) in enumerate(self.carried):
            c.carried_config[k] = _abi.WsCarriedConfig(decay, per_joule, min_speed)
        c.west_open, c.east_open = int(self.west_open), int(self.east_open)
        c.south_open, c.north_open = int(self.south_open), int(self.north_open)
        c.device = self.device
        return c


class Solver:
    """One rectangle of water, the reference's complete step on a GB300."""

    def __init__(self, config: Config):
        self.error = ""
        self._buf = C.create_string_buffer(512)
        self._h = None
        self.config = config
        h = C.c_void_p()
        if lib().ws_create(C.byref(config.to_c()), C.byref(h), self._buf, len(self._buf)) != 0:
            raise RuntimeError(self._buf.value.decode())
        self._h = h
        self._uploaded = {}  # input slot -> the array last uploaded (None: empty)

    def close(self):
        if self._h is not None:
            lib().ws_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def cells(self) -> int:
        return self.config.nx * self.config.ny

    def _check(self, rc):
        if rc != 0:
            self.error = self._buf.value.decode()
            raise RuntimeError(self.error)

    def _size(self, name):
        return self.cells * (len(self.config.carried) if name == "carried" else 1)

    # -- fields ------------------------------------------------------------------------------
    def set(self, name, values):
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        self._check(lib().ws_write_field(self._h, FIELDS[name], v.ctypes.data_as(_dp), v.size,
                                         self._buf, len(self._buf)))

    def get(self, name):
        out = np.zeros(self._size(name))
        if out.size:
            self._check(lib().ws_read_field(self._h, FIELDS[name], out.ctypes.data_as(_dp),
                                            out.size, self._buf, len(self._buf)))
        return out

    def depth(self):
        return self.get("depth")

    def momentum_x(self):
        return self.get("momentum_x")

    def momentum_y(self):
        return self.get("momentum_y")

    def ground(self):
        return self.get("ground")

    def carried(self, k):
        return self.get("carried")[k * self.cells:(k + 1) * self.cells]

    # -- inputs ------------------------------------------------------------------------------
    def set_input(self, slot: int, values):
        if values is None:
            rc = lib().ws_set_input(self._h, slot, None, 0, self._buf, len(self._buf))
        else:
            v = np.ascontiguousarray(values, dtype=np.float64).ravel()
            rc = lib().ws_set_input(self._h, slot, v.ctypes.data_as(_dp), v.size, self._buf,
                                    len(self._buf))
        self._check(rc)

    def set_inputs(self, inputs: dict):
        """The Inputs spans, uploaded where they differ from the last upload."""
        want = {INPUTS[k]: inputs.get(k) for k in INPUTS}
        nk = len(self.config.carried)
        for off, key in ((CARRIED_SOURCE, "carried_source"), (CARRIED_EXCHANGE, "carried_exchange")):
            arrays = list(inputs.get(key) or ())
            for k in range(nk):
                want[off + k] = arrays[k] if k < len(arrays) else None
        for slot, a in want.items():
            old = self._uploaded.get(slot, "unset")
            same = (a is None and old is None) or (
                a is not None and old is not None and not isinstance(old, str) and
                old.shape == np.shape(a) and np.array_equal(old, a))
            if not same:
                self.set_input(slot, a)
                self._uploaded[slot] = None if a is None else np.array(a, dtype=np.float64)

    # -- stepping ----------------------------------------------------------------------------
    def stable_step(self) -> float:
        return float(lib().ws_stable_step(self._h, self._buf, len(self._buf)))

    def step(self, inputs: dict, max_dt: float) -> float:
        self.set_inputs(inputs)
        return float(lib().ws_step(self._h, float(max_dt), self._buf, len(self._buf)))

    def advance(self, inputs: dict, duration_s: float) -> int:
        self.set_inputs(inputs)
        return int(lib().ws_advance(self._h, float(duration_s), self._buf, len(self._buf)))

    def run_steps(self, count: int, max_dt: float):
        self._check(lib().ws_run_steps(self._h, int(count), float(max_dt), self._buf,
                                       len(self._buf)))

    def enqueue_steps(self, stream, count: int, max_dt: float) -> bool:
        return lib().ws_enqueue_steps(self._h, stream, int(count), float(max_dt)) == 0

    def stream(self):
        return lib().ws_stream(self._h)

    # -- the account -------------------------------------------------------------------------
    def ledger(self) -> dict:
        out = _abi.WsLedger()
        self._check(lib().ws_read_ledger(self._h, C.byref(out), self._buf, len(self._buf)))
        d = {k: getattr(out, k) for k in LEDGER_KEYS}
        d["steps"] = int(d["steps"])
        d["carried"] = [{k: getattr(out.carried[q], k) for k in CARRIED_LEDGER_KEYS}
                        for q in range(len(self.config.carried))]
        return d

    def reset_ledger(self):
        self._check(lib().ws_reset_ledger(self._h, self._buf, len(self._buf)))

    def surface_volume_m3(self) -> float:
        return float(lib().ws_surface_volume_m3(self._h, self._buf, len(self._buf)))

    def ground_volume_m3(self) -> float:
        return float(lib().ws_ground_volume_m3(self._h, self._buf, len(self._buf)))

    def carried_total(self, k: int) -> float:
        return float(lib().ws_carried_total(self._h, int(k), self._buf, len(self._buf)))

    def state_hash(self) -> int:
        return int(lib().ws_state_hash(self._h, self._buf, len(self._buf)))

    def device_bytes(self) -> int:
        return int(lib().ws_device_bytes(self._h))

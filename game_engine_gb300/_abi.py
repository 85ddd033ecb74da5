"""ctypes declarations of include/wlcuda.h (the C ABI), kept beside the header's order."""
from __future__ import annotations

import ctypes as C

wl_stream = C.c_void_p
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_err = [C.c_char_p, C.c_size_t]


class Config(C.Structure):
    """wl_config: water_state::Config's fields the step reads (water_state.h:83-99)."""
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("cell_m", C.c_double),
                ("gravity", C.c_double), ("cfl", C.c_double), ("dry_depth_m", C.c_double),
                ("west_open", C.c_uint8), ("east_open", C.c_uint8), ("south_open", C.c_uint8),
                ("north_open", C.c_uint8), ("device", C.c_int32)]


class Options(C.Structure):
    """wl_options: StepOptions (water_live.h:105-110)."""
    _fields_ = [("ops", C.c_uint8), ("stored_faces", C.c_uint8)]


class StepParams(C.Structure):
    """wl_step_params: StepParams (water_live.h:66-88), 120 bytes."""
    _fields_ = [("state_in", C.c_uint64), ("state_out", C.c_uint64), ("bed", C.c_uint64),
                ("manning", C.c_uint64), ("source", C.c_uint64), ("partials", C.c_uint64),
                ("ledger", C.c_uint64), ("nx", C.c_uint32), ("ny", C.c_uint32),
                ("groups_x", C.c_uint32), ("group_count", C.c_uint32), ("flags", C.c_uint32),
                ("cell_m", C.c_float), ("gravity", C.c_float), ("cfl", C.c_float),
                ("dry_depth_m", C.c_float), ("max_dt", C.c_float), ("source_scale", C.c_float),
                ("pad", C.c_uint32), ("faces_x", C.c_uint64), ("faces_y", C.c_uint64)]


class Partial(C.Structure):
    """wl_partial: WaterPartial (water_live.h:114-121), 32 bytes."""
    _fields_ = [("speed_x", C.c_float), ("speed_y", C.c_float), ("source_m3", C.c_float),
                ("open_m3", C.c_float), ("roundoff_m3", C.c_float), ("pad", C.c_float * 3)]


class LedgerBits(C.Structure):
    """wl_ledger_bits: WaterLedger (water_live.h:124-137), 48 bytes."""
    _fields_ = [("time_hi", C.c_float), ("time_lo", C.c_float), ("source_hi", C.c_float),
                ("source_lo", C.c_float), ("open_hi", C.c_float), ("open_lo", C.c_float),
                ("roundoff_hi", C.c_float), ("roundoff_lo", C.c_float),
                ("remaining_s", C.c_float), ("dt", C.c_float), ("steps", C.c_uint32),
                ("pad", C.c_uint32)]


class Ledger(C.Structure):
    """wl_ledger: water_live::Ledger (water_live.h:143-150)."""
    _fields_ = [("source_m3", C.c_double), ("open_edge_out_m3", C.c_double),
                ("roundoff_m3", C.c_double), ("time_s", C.c_double),
                ("remaining_s", C.c_double), ("steps", C.c_uint64)]


class Tile(C.Structure):
    """wl_tile: one tile of a batch."""
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("west_open", C.c_uint8),
                ("east_open", C.c_uint8), ("south_open", C.c_uint8), ("north_open", C.c_uint8)]


class Tuning(C.Structure):
    """wl_tuning: the batched launch's shape."""
    _fields_ = [("block_rows", C.c_uint32), ("order", C.c_uint32), ("us_per_tick", C.c_float),
                ("zero_apart", C.c_uint32), ("stage", C.c_uint32)]


class Event(C.Structure):
    """wl_event: a rectangle of one plane a queued tick replaces."""
    _fields_ = [("kind", C.c_uint32), ("x0", C.c_uint32), ("y0", C.c_uint32), ("w", C.c_uint32),
                ("h", C.c_uint32), ("tile", C.c_uint32)]


class Landed(C.Structure):
    """wl_landed: a landed tick's read-back record."""
    _fields_ = [("tick", C.c_uint32), ("substeps", C.c_uint32), ("shortest_s", C.c_float),
                ("longest_s", C.c_float), ("time_hi", C.c_float), ("time_lo", C.c_float),
                ("steps", C.c_uint32), ("events", C.c_uint32), ("dropped", C.c_uint32),
                ("dropped_total", C.c_uint32), ("lag", C.c_uint32), ("frozen", C.c_uint32)]


class QueueStatus(C.Structure):
    """wl_queue_status: the queue's counts."""
    _fields_ = [("pushed", C.c_uint32), ("begun", C.c_uint32), ("landed", C.c_uint32),
                ("active", C.c_uint32), ("substeps", C.c_uint32), ("dropped", C.c_uint32),
                ("frozen", C.c_uint32), ("freezes", C.c_uint32)]


class WsCarriedConfig(C.Structure):
    """ws_carried_config: water_state::CarriedConfig (water_state.h:66-78)."""
    _fields_ = [("decay_s", C.c_double), ("per_joule", C.c_double),
                ("min_speed_m_per_s", C.c_double)]


class WsConfig(C.Structure):
    """ws_config: water_state::Config (water_state.h:83-99)."""
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("cell_m", C.c_double),
                ("gravity", C.c_double), ("cfl", C.c_double), ("dry_depth_m", C.c_double),
                ("water_density", C.c_double), ("carried", C.c_uint32), ("pad", C.c_uint32),
                ("carried_config", WsCarriedConfig * 4), ("west_open", C.c_uint8),
                ("east_open", C.c_uint8), ("south_open", C.c_uint8), ("north_open", C.c_uint8),
                ("device", C.c_int32)]


class WsCarriedLedger(C.Structure):
    _fields_ = [("source", C.c_double), ("from_dissipation", C.c_double),
                ("exchange", C.c_double), ("decayed", C.c_double), ("open_edge_out", C.c_double)]


class WsLedger(C.Structure):
    """ws_ledger: water_state::Ledger (water_state.h:135-145)."""
    _fields_ = [("source_m3", C.c_double), ("open_edge_out_m3", C.c_double),
                ("ground_m3", C.c_double), ("roundoff_m3", C.c_double),
                ("scheme_loss_j", C.c_double), ("friction_work_j", C.c_double),
                ("time_s", C.c_double), ("steps", C.c_uint64), ("carried", WsCarriedLedger * 4)]


_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)

# name -> (restype, argtypes); every symbol include/wlcuda.h declares.
SIGNATURES = {
    "wl_create": (C.c_int, [C.POINTER(Config), C.POINTER(Options), C.POINTER(C.c_void_p), *_err]),
    "wl_destroy": (None, [C.c_void_p]),
    "wl_valid": (C.c_int, [C.c_void_p]),
    "wl_cell_count": (C.c_uint32, [C.c_void_p]),
    "wl_group_count": (C.c_uint32, [C.c_void_p]),
    "wl_tick_launches": (C.c_uint64, [C.c_void_p]),
    "wl_staged_tiles": (C.c_uint32, [C.c_void_p]),
    "wl_resident_barrier_check": (C.c_int, [C.c_int, C.c_uint32, C.c_char_p, C.c_size_t]),
    "wl_write_state": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_size_t, *_err]),
    "wl_read_state": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_size_t, *_err]),
    "wl_read_state_bits": (C.c_int, [C.c_void_p, _fp, C.c_size_t, *_err]),
    "wl_read_ledger": (C.c_int, [C.c_void_p, C.POINTER(Ledger), *_err]),
    "wl_settled": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_size_t, C.c_float, C.c_float,
                             C.POINTER(C.c_uint8), C.POINTER(C.c_float), C.POINTER(C.c_float),
                             *_err]),
    "wl_set_bed": (C.c_int, [C.c_void_p, _dp, C.c_size_t, C.c_double, *_err]),
    "wl_set_manning": (C.c_int, [C.c_void_p, _dp, C.c_size_t, *_err]),
    "wl_set_source": (C.c_int, [C.c_void_p, _dp, C.c_size_t, C.c_uint32, C.c_int, *_err]),
    "wl_enqueue_steps": (C.c_int, [C.c_void_p, wl_stream, C.c_uint32, C.c_float]),
    "wl_run_steps": (C.c_int, [C.c_void_p, C.c_uint32, C.c_float, *_err]),
    "wl_advance": (C.c_uint64, [C.c_void_p, C.c_double, *_err]),
    "wl_state_hash": (C.c_uint64, [C.c_void_p, *_err]),
    "wl_read_partials_bits": (C.c_int, [C.c_void_p, C.POINTER(Partial), C.c_size_t, *_err]),
    "wl_read_ledger_bits": (C.c_int, [C.c_void_p, C.POINTER(LedgerBits), *_err]),
    "wl_run_length_pass": (C.c_int, [C.c_void_p, C.c_float, *_err]),
    "wl_hash_floats": (C.c_uint64, [_fp, C.c_size_t]),
    "wl_step_stream": (wl_stream, [C.c_void_p]),
    "wl_write_state_device": (C.c_int, [C.c_void_p, C.c_void_p, wl_stream]),
    "wl_device_planes": (C.c_int, [C.c_void_p, C.POINTER(_fp), C.POINTER(_fp), *_err]),
    "wl_batch_create": (C.c_int, [C.POINTER(Config), C.POINTER(Options), C.POINTER(Tile),
                                  C.c_uint32, C.POINTER(C.c_void_p), *_err]),
    "wl_batch_destroy": (None, [C.c_void_p]),
    "wl_batch_tile_count": (C.c_uint32, [C.c_void_p]),
    "wl_batch_cell_count": (C.c_uint64, [C.c_void_p]),
    "wl_batch_staged_tiles": (C.c_uint32, [C.c_void_p]),
    "wl_batch_tile_first": (C.c_uint64, [C.c_void_p, C.c_uint32]),
    "wl_batch_settled": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_size_t, C.c_float, C.c_float,
                                   C.POINTER(C.c_uint8), C.POINTER(C.c_float),
                                   C.POINTER(C.c_float), C.c_uint32, *_err]),
    "wl_batch_write_tile_state": (C.c_int, [C.c_void_p, C.c_uint32, _dp, _dp, _dp, C.c_size_t,
                                            *_err]),
    "wl_batch_write_state": (C.c_int, [C.c_void_p, _dp, _dp, _dp, C.c_size_t, *_err]),
    "wl_batch_set_bed": (C.c_int, [C.c_void_p, _dp, C.c_size_t, C.c_double, *_err]),
    "wl_batch_set_manning": (C.c_int, [C.c_void_p, _dp, C.c_size_t, *_err]),
    "wl_batch_set_source": (C.c_int, [C.c_void_p, _dp, C.c_size_t, C.c_uint32, C.c_int, *_err]),
    "wl_batch_enqueue_ticks": (C.c_int, [C.c_void_p, wl_stream, C.c_uint32, C.c_float]),
    "wl_batch_run_ticks": (C.c_int, [C.c_void_p, C.c_uint32, C.c_float, C.c_int, *_err]),
    "wl_batch_enqueue_tile_tick": (C.c_int, [C.c_void_p, wl_stream, C.c_uint32, C.c_float]),
    "wl_batch_run_tile_ticks": (C.c_int, [C.c_void_p, C.c_uint32, C.c_float, C.c_int,
                                          C.c_uint32, *_err]),
    "wl_batch_read_tile_bits": (C.c_int, [C.c_void_p, C.c_uint32, _fp, C.c_size_t, *_err]),
    "wl_batch_read_all_bits": (C.c_int, [C.c_void_p, _fp, C.c_size_t, *_err]),
    "wl_batch_tile_hash": (C.c_uint64, [C.c_void_p, C.c_uint32, *_err]),
    "wl_batch_tile_hashes": (C.c_int, [C.c_void_p, _u64p, C.c_uint32, *_err]),
    "wl_batch_read_ledgers": (C.c_int, [C.c_void_p, C.POINTER(Ledger), C.c_uint32, *_err]),
    "wl_batch_autotune": (C.c_int, [C.c_void_p, C.c_float, C.c_uint32, C.POINTER(Tuning), *_err]),
    "wl_batch_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning), *_err]),
    "wl_batch_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "wl_batch_stream": (wl_stream, [C.c_void_p]),
    "wl_util_fbm": (C.c_int, [_dp, C.c_uint32, C.c_uint32, C.c_double, C.c_uint64, C.c_uint32]),
    # the adjoint
    "wl_adjoint_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, _u32p, _dp,
                                    C.POINTER(C.c_void_p), *_err]),
    "wl_batch_adjoint_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, _u32p, _u32p, _dp,
                                          C.POINTER(C.c_void_p), *_err]),
    "wl_adjoint_destroy": (None, [C.c_void_p]),
    "wl_adjoint_enqueue": (C.c_int, [C.c_void_p, C.c_float]),
    "wl_adjoint_run": (C.c_int, [C.c_void_p, C.c_float, C.c_int, *_err]),
    "wl_adjoint_read": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _u32p, *_err]),
    "wl_adjoint_read_final": (C.c_int, [C.c_void_p, _fp, *_err]),
    "wl_adjoint_read_state_gradient": (C.c_int, [C.c_void_p, _fp, *_err]),
    "wl_adjoint_launches": (C.c_uint32, [C.c_void_p]),
    "wl_adjoint_device_bytes": (C.c_uint64, [C.c_void_p]),
    # one tick that allocates nothing
    "wl_tick_noalloc": (C.c_int, [C.POINTER(Config), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_float, wl_stream, *_err]),
    # the tick queue
    "wl_queue_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                  C.POINTER(C.c_void_p), *_err]),
    "wl_queue_destroy": (None, [C.c_void_p]),
    "wl_batch_queue_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                        C.POINTER(C.c_void_p), *_err]),
    "wl_queue_push": (C.c_int, [C.c_void_p, C.c_uint32, C.c_float, C.POINTER(Event), C.c_uint32,
                                _fp, C.c_size_t, *_err]),
    "wl_queue_enqueue_slots": (C.c_int, [C.c_void_p, wl_stream, C.c_uint32]),
    "wl_queue_set_limits": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, *_err]),
    "wl_queue_run_slots": (C.c_int, [C.c_void_p, C.c_uint32, *_err]),
    "wl_queue_status_read": (C.c_int, [C.c_void_p, C.POINTER(QueueStatus), *_err]),
    "wl_queue_read_landed": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(Landed),
                                       *_err]),
    "wl_queue_launches_per_slot": (C.c_uint32, []),
    "wl_queue_device_bytes": (C.c_uint64, [C.c_void_p]),
    # the complete FP64 step
    "ws_create": (C.c_int, [C.POINTER(WsConfig), C.POINTER(C.c_void_p), *_err]),
    "ws_destroy": (None, [C.c_void_p]),
    "ws_valid": (C.c_int, [C.c_void_p]),
    "ws_cell_count": (C.c_uint32, [C.c_void_p]),
    "ws_write_field": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_size_t, *_err]),
    "ws_read_field": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_size_t, *_err]),
    "ws_set_input": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_size_t, *_err]),
    "ws_stable_step": (C.c_double, [C.c_void_p, *_err]),
    "ws_step": (C.c_double, [C.c_void_p, C.c_double, *_err]),
    "ws_enqueue_steps": (C.c_int, [C.c_void_p, wl_stream, C.c_uint32, C.c_double]),
    "ws_run_steps": (C.c_int, [C.c_void_p, C.c_uint32, C.c_double, *_err]),
    "ws_advance": (C.c_uint64, [C.c_void_p, C.c_double, *_err]),
    "ws_read_ledger": (C.c_int, [C.c_void_p, C.POINTER(WsLedger), *_err]),
    "ws_reset_ledger": (C.c_int, [C.c_void_p, *_err]),
    "ws_surface_volume_m3": (C.c_double, [C.c_void_p, *_err]),
    "ws_ground_volume_m3": (C.c_double, [C.c_void_p, *_err]),
    "ws_carried_total": (C.c_double, [C.c_void_p, C.c_uint32, *_err]),
    "ws_state_hash": (C.c_uint64, [C.c_void_p, *_err]),
    "ws_stream": (wl_stream, [C.c_void_p]),
    "ws_device_bytes": (C.c_uint64, [C.c_void_p]),
}


def bind(lib: C.CDLL) -> C.CDLL:
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name, None)
        if f is None:
            continue  # a symbol check is the tests' job (tests/test_abi.py)
        f.restype = res
        f.argtypes = args
    return lib

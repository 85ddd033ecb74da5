"""The C ABI without a device: every symbol include/wlcuda.h declares is exported, the mirrored
structs keep the reference's sizes and offsets, the hash is FNV-1a, and a handle that was never
created refuses every call (water_live_tests.cpp:22-55).
"""
from __future__ import annotations

import ctypes as C
import json
import os
import re

import numpy as np

from game_engine_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PINS = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_pins.json")))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b((?:wl|ws)_\w*)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(wl_lib):
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(wl_lib, n)]
    assert not missing, missing
    # and the Python declarations cover them
    assert names <= set(_abi.SIGNATURES), sorted(names - set(_abi.SIGNATURES))


def test_sizes_and_offsets_are_the_reference_s():
    assert C.sizeof(_abi.StepParams) == PINS["sizes"]["StepParams"]
    assert C.sizeof(_abi.Partial) == PINS["sizes"]["WaterPartial"]
    assert C.sizeof(_abi.LedgerBits) == PINS["sizes"]["WaterLedger"]
    off = PINS["offsets"]
    for key, want in off.items():
        if key == "source":
            continue
        struct, field = key.split(".")
        cls = {"StepParams": _abi.StepParams, "WaterPartial": _abi.Partial,
               "WaterLedger": _abi.LedgerBits}[struct]
        assert getattr(cls, field).offset == want, key


def test_hash_is_fnv1a_over_float_bytes(wl_lib, oracle_mod):
    assert wl_lib.wl_hash_floats(None, 0) == int(PINS["fnv_empty"]["hash"])
    rng = np.random.default_rng(7)
    v = rng.standard_normal(1001).astype(np.float32)
    p = v.ctypes.data_as(C.POINTER(C.c_float))
    assert wl_lib.wl_hash_floats(p, v.size) == oracle_mod.hash_floats(v)
    w = v.copy()
    w.view(np.uint32)[500] ^= 1
    assert wl_lib.wl_hash_floats(w.ctypes.data_as(C.POINTER(C.c_float)), w.size) != \
        wl_lib.wl_hash_floats(p, v.size)


def test_a_step_never_created_refuses_every_call(wl_lib):
    # water_live_tests.cpp:38-47; WL_ERR_INVALID = 1, and 0 for the uint64 calls.
    from game_engine_gb300 import water_live as wl
    step = wl.DeviceStep()
    one = np.zeros(1)
    assert not step.valid()
    assert not step.set_bed(one, 0.0)
    assert not step.run_steps(1, 1.0)
    assert step.advance(1.0) == 0
    assert step.state_hash() == 0
    err = C.create_string_buffer(128)
    assert wl_lib.wl_valid(None) == 0
    assert wl_lib.wl_run_steps(None, 1, 1.0, err, 128) == 1
    assert b"no device" in err.value
    assert wl_lib.wl_write_state(None, None, None, None, 0, err, 128) == 1
    assert wl_lib.wl_read_ledger(None, None, err, 128) == 1
    assert wl_lib.wl_enqueue_steps(None, None, 1, 1.0) == 1
    assert wl_lib.wl_cell_count(None) == 0
    wl_lib.wl_destroy(None)


def test_an_empty_grid_is_refused(wl_lib):
    # water_live.cpp:108, before any device is touched
    cfg = _abi.Config(0, 4, 1.0, 9.81, 0.45, 1e-9, 0, 0, 0, 0, 0)
    out = C.c_void_p()
    err = C.create_string_buffer(128)
    assert wl_lib.wl_create(C.byref(cfg), None, C.byref(out), err, 128) == 2
    assert b"empty grid" in err.value
    assert not out.value
    # A tile's cells are indexed in 32 bits: more than 2^30 cells is refused the same way.
    big = _abi.Config(32768, 32769, 1.0, 9.81, 0.45, 1e-9, 0, 0, 0, 0, 0)
    assert wl_lib.wl_create(C.byref(big), None, C.byref(out), err, 128) == 2
    assert b"2^30" in err.value and not out.value


def test_the_numerics_policy_of_every_build():
    # The reference's contraction sanitizer (water_live_tests.cpp:57-105) checks its SPIR-V for
    # contracted float operations. Here the same policy is held at the build: every translation
    # unit of the tick compiles with no contraction and IEEE division and square root, the host
    # code and the oracle with -ffp-contract=off. The adjoint's unit alone takes contraction (its
    # reverse march is a derivative held to a tolerance; its forward is spelled in _rn intrinsics).
    from game_engine_gb300 import buildlib
    for src in buildlib.SOURCES:
        flags = buildlib.NUMERICS_BY_SOURCE.get(src, buildlib.NUMERICS)
        assert "-prec-div=true" in flags and "-prec-sqrt=true" in flags and "-ftz=false" in flags
        if src != "wl_adjoint.cu":
            assert "--fmad=false" in flags, src
    assert "-ffp-contract=off" in ",".join(buildlib.HOST)
    make = open(os.path.join(ROOT, "oracle", "Makefile")).read()
    assert "-ffp-contract=off" in make and "-fno-fast-math" in make
    # the adjoint's forward march spells every + - * / of the update in correctly rounded
    # intrinsics: no bare float operator on its lines
    src = open(os.path.join(ROOT, "game_engine_gb300", "csrc", "wl_adjoint.cu")).read()
    fwd = src[src.index("__device__ void forward_march("):src.index("// ---- the reverse march")]
    update = fwd[fwd.index("float h = __fsub_rn("):fwd.index("out[i] = h;")]
    code = re.sub(r"//[^\n]*", "", update)
    assert not re.search(r"[\w)\]]\s*[-+*/]\s*[\w(]", re.sub(r"__f\w+_rn\(|\b\d+\.\d+f\b", "", code)
                         .replace("-added", "").replace("-target", "")), "a bare float operator"


def test_a_queue_without_a_step_refuses_every_call(wl_lib):
    # The tick queue's calls with no step or no queue: WL_ERR_INVALID (1), nothing touched.
    err = C.create_string_buffer(128)
    out = C.c_void_p()
    assert wl_lib.wl_queue_create(None, 64, 1024, 16, C.byref(out), err, 128) == 1
    assert not out.value
    assert wl_lib.wl_queue_create(None, 64, 1024, 16, None, err, 128) == 8
    assert wl_lib.wl_queue_push(None, 0, 0.01, None, 0, None, 0, err, 128) == 1
    assert wl_lib.wl_queue_enqueue_slots(None, None, 4) == 1
    assert wl_lib.wl_queue_run_slots(None, 4, err, 128) == 1
    assert wl_lib.wl_queue_status_read(None, None, err, 128) == 1
    assert wl_lib.wl_queue_read_landed(None, 0, 1, None, err, 128) == 1
    assert wl_lib.wl_queue_launches_per_slot() == 2
    assert wl_lib.wl_queue_device_bytes(None) == 0
    wl_lib.wl_queue_destroy(None)


def test_a_full_solver_never_created_refuses_every_call(wl_lib):
    # The complete FP64 step's calls with no solver: WL_ERR_INVALID (1), 0 for the value calls.
    err = C.create_string_buffer(128)
    assert wl_lib.ws_valid(None) == 0
    assert wl_lib.ws_cell_count(None) == 0
    assert wl_lib.ws_write_field(None, 0, None, 0, err, 128) == 1
    assert wl_lib.ws_set_input(None, 0, None, 0, err, 128) == 1
    assert wl_lib.ws_step(None, 0.1, err, 128) == 0.0
    assert wl_lib.ws_advance(None, 1.0, err, 128) == 0
    assert wl_lib.ws_enqueue_steps(None, None, 1, 0.1) == 1
    assert wl_lib.ws_state_hash(None, err, 128) == 0
    assert wl_lib.ws_read_ledger(None, None, err, 128) == 1
    wl_lib.ws_destroy(None)
    cfg = _abi.WsConfig()
    cfg.nx, cfg.ny = 0, 4
    out = C.c_void_p()
    assert wl_lib.ws_create(C.byref(cfg), C.byref(out), err, 128) == 2 and not out.value
    cfg.nx, cfg.carried = 4, 5
    assert wl_lib.ws_create(C.byref(cfg), C.byref(out), err, 128) == 8 and not out.value
    assert C.sizeof(_abi.WsConfig) == 160 and C.sizeof(_abi.WsLedger) == 224


def test_an_adjoint_never_created_refuses_every_read(wl_lib):
    # The sweep's read-backs with no sweep: WL_ERR_INVALID (1); 0 for the count calls.
    err = C.create_string_buffer(128)
    buf = (C.c_float * 3)()
    assert wl_lib.wl_adjoint_read(None, None, None, None, None, err, 128) == 1
    assert wl_lib.wl_adjoint_read_final(None, buf, err, 128) == 1
    assert wl_lib.wl_adjoint_read_state_gradient(None, buf, err, 128) == 1
    assert b"no sweep" in err.value
    assert wl_lib.wl_adjoint_launches(None) == 0
    assert wl_lib.wl_adjoint_device_bytes(None) == 0
    wl_lib.wl_adjoint_destroy(None)


def test_a_batch_with_an_empty_or_oversized_tile_is_refused(wl_lib):
    # Before any device is touched: an empty tile, or one of more than 2^30 cells.
    cfg = _abi.Config(0, 0, 1.0, 9.81, 0.45, 1e-9, 0, 0, 0, 0, 0)
    out = C.c_void_p()
    err = C.create_string_buffer(128)
    tiles = (_abi.Tile * 2)(_abi.Tile(64, 64, 0, 0, 0, 0), _abi.Tile(0, 8, 0, 0, 0, 0))
    assert wl_lib.wl_batch_create(C.byref(cfg), None, tiles, 2, C.byref(out), err, 128) == 2
    assert b"empty grid" in err.value and not out.value
    tiles[1] = _abi.Tile(40000, 40000, 0, 0, 0, 0)
    assert wl_lib.wl_batch_create(C.byref(cfg), None, tiles, 2, C.byref(out), err, 128) == 2
    assert b"2^30" in err.value and not out.value
    assert wl_lib.wl_batch_create(C.byref(cfg), None, tiles, 0, C.byref(out), err, 128) == 2

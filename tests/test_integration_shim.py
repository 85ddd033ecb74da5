"""The engine-side bindings, compiled as a maintainer would use them: include/wlcuda_device_step.hpp
(water_live::DeviceStep's method set over the C ABI) and include/wlcuda_solver.hpp (the complete
FP64 step's water_state::Solver), each against the reference's own water_state.h, linked to
libwlcuda.so and run on the CPU.

- The DeviceStep binding compiles against a stand-in water_live.h that declares only the PODs it
  uses, mirrored from water_live.h:57-150 (tests/shim_include; the engine's own header pulls in the
  gfx layer, whose generated code the reference's tree does not hold). Its layouts are held to the
  C ABI's, and without a device every call through it refuses: create fails with the library's
  message, valid() is false, the hash and advance return 0, misfit spans are refused before any
  call, and hash_floats of nothing is FNV-1a's offset basis (water_live_tests.cpp:49-55).
- The Solver binding's ledger, carried ledger and carried config have the reference's layouts field
  by field, and without a device every call through it refuses.

The reference's headers are found through oracle.reference_root(); the test skips where they are
absent.
"""
from __future__ import annotations

import os
import subprocess

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = oracle.reference_root()
needs_ref = pytest.mark.skipif(
    REF is None or not os.path.isdir(os.path.join(REF, "domain", "water_state")),
    reason="the reference's sources are not here")

DEVICE_STEP_MAIN = r'''
#include "wlcuda_device_step.hpp"

#include <cstdio>
#include <vector>

using namespace engine;

static_assert(sizeof(water_live::WaterPartial) == sizeof(wl_partial), "WaterPartial");
static_assert(sizeof(water_live::WaterLedger) == sizeof(wl_ledger_bits), "WaterLedger");
static_assert(sizeof(water_live::Ledger) == sizeof(wl_ledger), "Ledger");

int main() {
  water_state::Config c;
  c.nx = 8;
  c.ny = 4;
  c.edges.east = water_state::Edge::open;
  water_live::StepOptions o;
  o.ops = water_live::Ops::fixed;
  water_live_cuda::DeviceStep s;
  std::string err;
  const bool made = s.create(0, c, o, &err);
  std::vector<f64> h(32, 1.0), short_span(31, 0.0);
  std::string refused;
  const bool wrote = s.write_state(h, short_span, h, &refused);
  std::string hash_err;
  const u64 hash = s.state_hash(&hash_err);
  const u64 steps = s.advance(1.0);
  water_live::Ledger led;
  const bool read = s.read_ledger(led);
  const u64 empty = water_live_cuda::hash_floats({});
  std::printf("%d|%d|%d|%llu|%llu|%d|%llu|%s|%s|%d\n", made ? 1 : 0, s.valid() ? 1 : 0,
              wrote ? 1 : 0, static_cast<unsigned long long>(hash),
              static_cast<unsigned long long>(steps), read ? 1 : 0,
              static_cast<unsigned long long>(empty), refused.c_str(),
              err.empty() ? "-" : "message", hash_err.empty() ? 0 : 1);
  return 0;
}
'''

SOLVER_MAIN = r'''
#include "wlcuda_solver.hpp"

#include <cstddef>
#include <cstdio>

using namespace engine;

#define SAME(a, b, f) static_assert(offsetof(a, f) == offsetof(b, f), #f)
static_assert(sizeof(ws_ledger) == sizeof(water_state::Ledger), "Ledger size");
SAME(ws_ledger, water_state::Ledger, source_m3);
SAME(ws_ledger, water_state::Ledger, open_edge_out_m3);
SAME(ws_ledger, water_state::Ledger, ground_m3);
SAME(ws_ledger, water_state::Ledger, roundoff_m3);
SAME(ws_ledger, water_state::Ledger, scheme_loss_j);
SAME(ws_ledger, water_state::Ledger, friction_work_j);
SAME(ws_ledger, water_state::Ledger, time_s);
SAME(ws_ledger, water_state::Ledger, steps);
SAME(ws_ledger, water_state::Ledger, carried);
static_assert(sizeof(ws_carried_ledger) == sizeof(water_state::CarriedLedger), "CarriedLedger");
SAME(ws_carried_ledger, water_state::CarriedLedger, source);
SAME(ws_carried_ledger, water_state::CarriedLedger, from_dissipation);
SAME(ws_carried_ledger, water_state::CarriedLedger, exchange);
SAME(ws_carried_ledger, water_state::CarriedLedger, decayed);
SAME(ws_carried_ledger, water_state::CarriedLedger, open_edge_out);
static_assert(sizeof(ws_carried_config) == sizeof(water_state::CarriedConfig), "CarriedConfig");

int main() {
  water_state::Config c;
  c.nx = 8;
  c.ny = 4;
  c.carried = 1;
  water_state_cuda::Solver s(c, 0);
  f64 depth[32] = {};
  water_state::Inputs in;
  const bool wrote = s.write(WS_DEPTH, std::span<const f64>(depth, 32));
  const f64 dt = s.step(in, 0.01);
  std::printf("%d %d %g %llu\n", s.valid() ? 1 : 0, wrote ? 1 : 0, dt,
              static_cast<unsigned long long>(s.state_hash()));
  return 0;
}
'''


def _compile_and_run(tmp_path, name, source, extra_inc=()):
    from game_engine_gb300 import LIB_PATH
    src = tmp_path / f"{name}.cpp"
    src.write_text(source)
    inc = [f"-I{os.path.join(REF, 'core', d, 'include')}"
           for d in sorted(os.listdir(os.path.join(REF, "core")))
           if os.path.isdir(os.path.join(REF, "core", d, "include"))]
    inc += [f"-I{os.path.join(REF, 'domain', 'water_state', 'include')}",
            f"-I{os.path.join(ROOT, 'include')}"] + [f"-I{d}" for d in extra_inc]
    libdir = os.path.dirname(LIB_PATH)
    exe = tmp_path / name
    cmd = ["g++", "-std=c++20", "-O1", "-Wall", *inc, str(src), "-o", str(exe), f"-L{libdir}",
           "-lwlcuda", f"-Wl,-rpath,{libdir}", "-L/usr/local/cuda/lib64",
           "-Wl,-rpath,/usr/local/cuda/lib64", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stderr
    return run.stdout.strip()


def _has_device():
    import torch
    return torch.cuda.is_available()


@needs_ref
def test_the_device_step_shim_compiles_and_refuses_without_a_device(tmp_path, wl_lib):
    out = _compile_and_run(tmp_path, "device_step", DEVICE_STEP_MAIN,
                           [os.path.join(ROOT, "tests", "shim_include")])
    made, valid, wrote, h, steps, read, empty, refused, err, hash_err = out.split("|")
    assert wrote == "0" and refused == "water_live: spans of different sizes"
    assert int(empty) == 0xCBF29CE484222325
    if not _has_device():
        assert (made, valid, int(h), int(steps), read) == ("0", "0", 0, 0, "0")
        assert err == "message" and hash_err == "1"


@needs_ref
def test_the_solver_shim_compiles_against_the_reference(tmp_path, wl_lib):
    out = _compile_and_run(tmp_path, "solver", SOLVER_MAIN)
    valid, wrote, dt, h = out.split()
    if not _has_device():
        # Without a device the solver is never made: every call through the shim refuses.
        assert (valid, wrote, float(dt), int(h)) == ("0", "0", 0.0, 0)

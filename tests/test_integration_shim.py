"""The engine-side binding INTEGRATION.md shows for the complete FP64 step, compiled against the
reference's own water_state.h (where the reference's sources are present) and linked to
libwlcuda.so: the shim compiles as written, ws_ledger and ws_carried_ledger have
water_state::Ledger's and CarriedLedger's layout field by field, and without a device every call
through the shim refuses. (The DeviceStep shim of INTEGRATION.md section 1 includes the engine's
gfx headers, which need generated schema code that is not in the reference's tree.)
"""
from __future__ import annotations

import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"

MAIN = r'''
#include <domain/water_state/water_state.h>
#include "wlcuda.h"

#include <cstddef>
#include <cstdio>

using namespace engine;

#include "shim.hpp"

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
  std::printf("%d %g %llu\n", wrote ? 1 : 0, dt, static_cast<unsigned long long>(s.state_hash()));
  return 0;
}
'''


def shim_source():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    section = text[text.index("## 5. The complete FP64 step's shim"):]
    return re.search(r"```cpp\n(.*?)```", section, re.S).group(1)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "domain", "water_state")),
                    reason="the reference's sources are not here")
def test_the_solver_shim_compiles_against_the_reference(tmp_path, wl_lib):
    from game_engine_gb300 import LIB_PATH
    (tmp_path / "shim.hpp").write_text(shim_source())
    (tmp_path / "main.cpp").write_text(MAIN)
    inc = [f"-I{os.path.join(REF, 'core', d, 'include')}"
           for d in sorted(os.listdir(os.path.join(REF, "core")))
           if os.path.isdir(os.path.join(REF, "core", d, "include"))]
    inc += [f"-I{os.path.join(REF, 'domain', 'water_state', 'include')}",
            f"-I{os.path.join(ROOT, 'include')}", f"-I{tmp_path}"]
    libdir = os.path.dirname(LIB_PATH)
    exe = tmp_path / "shim"
    cmd = ["g++", "-std=c++20", "-O1", *inc, str(tmp_path / "main.cpp"), "-o", str(exe),
           f"-L{libdir}", "-lwlcuda", f"-Wl,-rpath,{libdir}", "-L/usr/local/cuda/lib64",
           "-Wl,-rpath,/usr/local/cuda/lib64", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stderr
    wrote, dt, h = run.stdout.split()
    # Without a device the solver is never made: every call through the shim refuses.
    assert (wrote, float(dt), int(h)) == ("0", 0.0, 0)

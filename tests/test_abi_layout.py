"""The ctypes mirrors in game_engine_gb300/_abi.py against include/wlcuda.h itself: a small C
program (gcc, no device) prints every mirrored struct's size and each field's offset, and each
must equal the ctypes layout, so a change on one side without the other fails here."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import pytest

from game_engine_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = {
    "wl_config": _abi.Config,
    "wl_options": _abi.Options,
    "wl_step_params": _abi.StepParams,
    "wl_partial": _abi.Partial,
    "wl_ledger_bits": _abi.LedgerBits,
    "wl_ledger": _abi.Ledger,
    "wl_tile": _abi.Tile,
    "wl_tuning": _abi.Tuning,
    "wl_event": _abi.Event,
    "wl_landed": _abi.Landed,
    "wl_queue_status": _abi.QueueStatus,
    "ws_carried_config": _abi.WsCarriedConfig,
    "ws_config": _abi.WsConfig,
    "ws_carried_ledger": _abi.WsCarriedLedger,
    "ws_ledger": _abi.WsLedger,
}


def c_layout():
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "wlcuda.h"', "int main(void) {"]
    for cname, cls in MIRRORS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for field, *_ in cls._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        with open(src, "w") as f:
            f.write("\n".join(lines) + "\n")
        subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe],
                       check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        cname, key, value = line.split()
        layout[(cname, key)] = int(value)
    return layout


@pytest.fixture(scope="module")
def layout():
    try:
        return c_layout()
    except (OSError, subprocess.CalledProcessError) as e:
        pytest.skip(f"no C compiler for the layout probe: {e}")


@pytest.mark.parametrize("cname", sorted(MIRRORS))
def test_ctypes_mirror_matches_the_header(layout, cname):
    cls = MIRRORS[cname]
    assert C.sizeof(cls) == layout[(cname, "sizeof")], cname
    for field, *_ in cls._fields_:
        assert getattr(cls, field).offset == layout[(cname, field)], f"{cname}.{field}"

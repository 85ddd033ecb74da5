"""Runs one case through the CUDA path (the C ABI) and through the oracle, side by side."""
from __future__ import annotations

import os
from contextlib import contextmanager

import numpy as np

import oracle
from game_engine_gb300 import water_live as wl


@contextmanager
def block_rows(rows):
    """The tick's block shape for steps created inside (WLCUDA_BLOCK_ROWS: 16, 32 or 64)."""
    old = os.environ.get("WLCUDA_BLOCK_ROWS")
    if rows is None:
        os.environ.pop("WLCUDA_BLOCK_ROWS", None)
    else:
        os.environ["WLCUDA_BLOCK_ROWS"] = str(rows)
    try:
        yield
    finally:
        if old is None:
            os.environ.pop("WLCUDA_BLOCK_ROWS", None)
        else:
            os.environ["WLCUDA_BLOCK_ROWS"] = old


def config(c):
    e = c.get("open_edges", 0)
    return wl.Config(c["nx"], c["ny"], c["cell_m"], west_open=bool(e & 1), east_open=bool(e & 2),
                     south_open=bool(e & 4), north_open=bool(e & 8))


def make_pair(c, fixed=False, every=1, compensate=False, datum=0.0, rows=None,
              stored_faces=False):
    """(device step, oracle step), both loaded with the case."""
    g = oracle.Grid(c["nx"], c["ny"], c["cell_m"], open_edges=c.get("open_edges", 0))
    ref = oracle.RefStep(g, fixed_ops=fixed)
    dev = wl.DeviceStep()
    with block_rows(rows):
        ok = dev.create(config(c), wl.StepOptions(ops=wl.OPS_FIXED if fixed else wl.OPS_NATIVE,
                                                  stored_faces=stored_faces))
    assert ok, dev.error
    n = g.cells
    hu = c.get("hu", np.zeros(n))
    hv = c.get("hv", np.zeros(n))
    for o in (ref, dev):
        o.set_bed(c["bed"], datum)
        if c.get("manning") is not None:
            o.set_manning(c["manning"])
        if c.get("source") is not None:
            o.set_source(c["source"], every, compensate)
    ref.write_state(c["h"], hu, hv)
    assert dev.write_state(c["h"], hu, hv), dev.error
    return dev, ref


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def assert_same(dev, ref, what=""):
    """The state's four planes, the records and the ledger's 48 bytes, bit for bit."""
    a = dev.read_state_bits()
    b = ref.read_state_bits()
    diff = np.nonzero(bits(a) != bits(b))[0]
    assert diff.size == 0, (f"{what}: {diff.size} state words differ, first at {diff[:5]}: "
                            f"{a[diff[:5]]} vs {b[diff[:5]]}")
    assert np.array_equal(bits(dev.read_partials_bits()), bits(ref.read_partials_bits())), \
        f"{what}: records differ"
    assert np.array_equal(dev.read_ledger_bits(), ref.read_ledger_bits()), f"{what}: ledger differs"
    assert dev.state_hash() == ref.state_hash()

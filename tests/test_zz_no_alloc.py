"""The allocation-free tick (wl_tick_noalloc): two calls in a row, each one tick of a state the
caller owns on the device, give the bytes the step's own entry point (wl_run_steps) gives for the
same two ticks; a grid past the scratch's limit is refused. Collected last, and passes alone."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import cases
from game_engine_gb300 import _abi, lib
from pairs import make_pair

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _tick(cfg, fixed, src, dst, bed, manning, source, max_dt, stream):
    buf = C.create_string_buffer(256)
    rc = lib().wl_tick_noalloc(C.byref(cfg), int(fixed), _ptr(src), _ptr(dst), _ptr(bed),
                               _ptr(manning) if manning is not None else None,
                               _ptr(source) if source is not None else None, float(max_dt),
                               C.c_void_p(stream), buf, len(buf))
    return rc, buf.value.decode()


@pytest.mark.parametrize("name,fixed", [("slope", False), ("slope", True), ("all_open", False),
                                        ("basin", False), ("lake", False)])
def test_two_ticks_in_a_row_equal_the_step(gpu, name, fixed):
    import torch
    c = {"slope": cases.slope(False), "all_open": cases.slope(True),
         "basin": cases.closed_basin(), "lake": cases.inexact_lake()}[name]
    dev, _ = make_pair(c, fixed=fixed)
    n = c["nx"] * c["ny"]
    f32 = lambda a: torch.from_numpy(np.asarray(a, dtype=np.float64).astype(np.float32)).cuda()
    in0 = torch.from_numpy(dev.read_state_bits()).cuda()
    out1 = torch.zeros_like(in0)
    out2 = torch.zeros_like(in0)
    bed = f32(c["bed"])
    manning = f32(c["manning"]) if c.get("manning") is not None else None
    source = f32(c["source"]) if c.get("source") is not None else None
    e = c.get("open_edges", 0)
    cfg = _abi.Config(c["nx"], c["ny"], c["cell_m"], 9.81, 0.45, 1e-9, e & 1, (e >> 1) & 1,
                      (e >> 2) & 1, (e >> 3) & 1, 0)
    stream = torch.cuda.current_stream().cuda_stream
    max_dt = 0.01
    for src, dst in ((in0, out1), (out1, out2)):
        rc, msg = _tick(cfg, fixed, src, dst, bed, manning, source, max_dt, stream)
        assert rc == 0, msg
    torch.cuda.synchronize()
    assert dev.run_steps(1, max_dt), dev.error
    want1 = dev.read_state_bits()
    assert dev.run_steps(1, max_dt), dev.error
    want2 = dev.read_state_bits()
    got1, got2 = out1.cpu().numpy(), out2.cpu().numpy()
    assert np.array_equal(got1[:3 * n].view(np.uint32), want1[:3 * n].view(np.uint32))
    assert np.array_equal(got2[:3 * n].view(np.uint32), want2[:3 * n].view(np.uint32))


def test_a_grid_past_the_limit_is_refused(gpu):
    import torch
    t = torch.zeros(4 * 16, device="cuda")
    cfg = _abi.Config(1040, 1024, 1.0, 9.81, 0.45, 1e-9, 0, 0, 0, 0, 0)  # 65 x 64 groups
    rc, msg = _tick(cfg, False, t, t[1:], t, None, None, 0.01, 0)
    assert rc == 2 and "at most 4096" in msg  # WL_ERR_SIZE, nothing launched
    cfg = _abi.Config(1024, 1024, 1.0, 9.81, 0.45, 1e-9, 0, 0, 0, 0, 0)
    rc, msg = _tick(cfg, False, t, t, t, None, None, 0.01, 0)
    assert rc == 8  # the same copy in and out: WL_ERR_ARGUMENT

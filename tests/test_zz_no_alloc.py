"""The allocation-free tick (wl_tick_noalloc), for callers that cannot allocate device memory: an
engine frame loop that reserved its memory at start, or a real-time thread that must not touch the
allocator. Two calls in a row, each one tick of a state the caller owns on the device, must give
the bytes the step's own entry point (wl_run_steps) gives for the same two ticks: all four planes,
bit for bit. The cases cover the small shapes (three-phase blocks), a grid of exactly the
scratch's 4096 groups of 16 x 16 and one of 4095 whose width is not a multiple of 32, and a long
thin grid that takes the 32 x 16 march with its last items a CTA at a time. A warmed-up loop of
calls leaves the device's free memory unchanged, and a grid past the limit is refused.

Collected last (its file name), so a run that stops at the first failure has run every other test
first; it passes alone in a fresh process as well."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import cases
from game_engine_gb300 import _abi, lib, workloads
from pairs import make_pair

pytestmark = pytest.mark.gpu

MAX_DT = 0.01


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _tick(cfg, fixed, src, dst, bed, manning, source, max_dt, stream):
    buf = C.create_string_buffer(256)
    rc = lib().wl_tick_noalloc(C.byref(cfg), int(fixed), _ptr(src), _ptr(dst), _ptr(bed),
                               _ptr(manning) if manning is not None else None,
                               _ptr(source) if source is not None else None, float(max_dt),
                               C.c_void_p(stream), buf, len(buf))
    return rc, buf.value.decode()


def _big(nx, ny, seed):
    """A seeded landscape: fBm relief under a lake whose surface has a bump, rain on every cell."""
    bed = workloads.fbm(nx, ny, 4.0, seed)
    x, y = np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64))
    surf = 2.5 + 0.8 * np.exp(-((x - 0.3 * nx) ** 2 + (y - 0.6 * ny) ** 2) / (0.01 * nx * ny + 9))
    h = np.maximum(surf.ravel() - bed, 0.0)
    return dict(nx=nx, ny=ny, cell_m=1.0, bed=bed, h=h, source=np.full(nx * ny, 2e-4))


def _case(name):
    return {"slope": lambda: cases.slope(False), "all_open": lambda: cases.slope(True),
            "basin": cases.closed_basin, "lake": cases.inexact_lake,
            "groups_4096": lambda: _big(1024, 1024, 71),
            "groups_4095": lambda: _big(1008, 1040, 72),
            "march_16x65536": lambda: _big(16, 65536, 73)}[name]()


def _setup(c, fixed):
    import torch
    dev, _ = make_pair(c, fixed=fixed)
    f32 = lambda a: torch.from_numpy(np.asarray(a, dtype=np.float64).astype(np.float32)).cuda()
    in0 = torch.from_numpy(dev.read_state_bits()).cuda()
    bed = f32(c["bed"])
    manning = f32(c["manning"]) if c.get("manning") is not None else None
    source = f32(c["source"]) if c.get("source") is not None else None
    e = c.get("open_edges", 0)
    cfg = _abi.Config(c["nx"], c["ny"], c["cell_m"], 9.81, 0.45, 1e-9, e & 1, (e >> 1) & 1,
                      (e >> 2) & 1, (e >> 3) & 1, 0)
    return dev, in0, bed, manning, source, cfg


@pytest.mark.parametrize("name,fixed", [("slope", False), ("slope", True), ("all_open", False),
                                        ("basin", False), ("lake", False),
                                        ("groups_4096", False), ("groups_4095", False),
                                        ("march_16x65536", False)])
def test_two_ticks_in_a_row_equal_the_step(gpu, name, fixed):
    import torch
    c = _case(name)
    dev, in0, bed, manning, source, cfg = _setup(c, fixed)
    out1 = torch.zeros_like(in0)
    out2 = torch.zeros_like(in0)
    stream = torch.cuda.current_stream().cuda_stream
    for src, dst in ((in0, out1), (out1, out2)):
        rc, msg = _tick(cfg, fixed, src, dst, bed, manning, source, MAX_DT, stream)
        assert rc == 0, msg
    torch.cuda.synchronize()
    assert dev.run_steps(1, MAX_DT), dev.error
    want1 = dev.read_state_bits()
    assert dev.run_steps(1, MAX_DT), dev.error
    want2 = dev.read_state_bits()
    got1, got2 = out1.cpu().numpy(), out2.cpu().numpy()
    # All four planes: h, hu, hv and the remainder (which a tick without the compensated source
    # leaves as the caller's zeros, as the step leaves its own).
    assert np.array_equal(got1.view(np.uint32), want1.view(np.uint32)), f"{name}: first tick"
    assert np.array_equal(got2.view(np.uint32), want2.view(np.uint32)), f"{name}: second tick"
    dev.destroy()


def test_a_loop_of_calls_takes_no_device_memory(gpu):
    import torch
    c = _case("groups_4096")
    dev, in0, bed, manning, source, cfg = _setup(c, False)
    dev.destroy()
    a, b = in0.clone(), torch.zeros_like(in0)
    stream = torch.cuda.current_stream().cuda_stream
    rc, msg = _tick(cfg, False, a, b, bed, manning, source, MAX_DT, stream)  # warm-up: set-up
    assert rc == 0, msg
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for k in range(20):
        src, dst = (a, b) if k % 2 == 0 else (b, a)
        rc, msg = _tick(cfg, False, src, dst, bed, manning, source, MAX_DT, stream)
        assert rc == 0, msg
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)


def test_a_grid_past_the_limit_is_refused(gpu):
    import torch
    t = torch.zeros(4 * 16, device="cuda")
    cfg = _abi.Config(1040, 1024, 1.0, 9.81, 0.45, 1e-9, 0, 0, 0, 0, 0)  # 65 x 64 groups
    rc, msg = _tick(cfg, False, t, t[1:], t, None, None, MAX_DT, 0)
    assert rc == 2 and "at most 4096" in msg  # WL_ERR_SIZE, nothing launched
    cfg = _abi.Config(16, 65552, 1.0, 9.81, 0.45, 1e-9, 0, 0, 0, 0, 0)  # 1 x 4097 groups
    rc, msg = _tick(cfg, False, t, t[1:], t, None, None, MAX_DT, 0)
    assert rc == 2 and "at most 4096" in msg
    cfg = _abi.Config(1024, 1024, 1.0, 9.81, 0.45, 1e-9, 0, 0, 0, 0, 0)
    rc, msg = _tick(cfg, False, t, t, t, None, None, MAX_DT, 0)
    assert rc == 8  # the same copy in and out: WL_ERR_ARGUMENT

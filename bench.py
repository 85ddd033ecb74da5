#!/usr/bin/env python3
"""Benchmark of the live-water tick on a GB300 (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload plain_2048|plain_256|plain_1024|tiles_4096|adjoint_512|
                               tiles_256_adjoint|tick_queue|full_step]

The metric is water cell-updates per second. A bench step is one pass of the workload over its
configuration: for the default (plain_2048, the throughput configuration) 500 ticks of one
2048 x 2048 tile from the same seeded initial state. `value` runs with the inputs resident in HBM
(each step restores the initial state from a device copy, untimed work between steps flushes L2);
`e2e` runs the same steps through the C ABI with host buffers: upload of the state, bed and source,
the ticks, and the read-back of the state, every step.

Beside the headline (unless --no-extras): `batched`, the 4096-tile configuration in one persistent
graph-captured launch a tick against the per-tile-launch form; `adjoint` and `batched_adjoint`, the
checkpointed sweep's seconds per tick (forward and reverse) against the plain tick's on the same
tiles; `tick_queue`, a captured frame of queue slots, busy and idle, against the plain tick;
`full_step`, the complete FP64 step (ground store, carried quantities, outputs) on the device
against the reference's CPU step restated in oracle/.

`--impl reference` times the reference's CPU tick (the FP64 solver, water_state::Solver::step,
restated in oracle/ and checked byte for byte against the reference's own build) on this host's
cores, on the same workload: the same ticks a step from the same initial state. Its process loads
the oracle's library only (the terrain comes from the numpy generator).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 512 << 20  # larger than the GB300's L2 (129 MB)
CONFIGS_GOLDEN = os.path.join(ROOT, "tests", "golden", "configs.json")


def golden_config(name):
    """The oracle's answer for a configuration at full size (tests/golden/make_configs.py), or
    None where the fixture is absent."""
    try:
        with open(CONFIGS_GOLDEN) as f:
            return json.load(f).get(name)
    except OSError:
        return None


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region (every 200 ms)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in self.file:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names[1:], parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------------------
# the reference's CPU tick (the oracle's FP64 restatement of water_state::Solver::step)

def cpu_baseline(tile, threads: int, budget_s: float = 12.0):
    """Times the reference CPU tick on `tile` with `threads` host threads; bounded sample."""
    import oracle  # the CPU baseline leg: the oracle's restatement of the reference CPU tick
    g = oracle.Grid(tile.nx, tile.ny, tile.cell_m)
    s = oracle.Solver64(g, threads)
    s.set_state(tile.h, tile.hu, tile.hv)
    s.set_inputs(tile.bed, None, tile.source)
    max_dt = tile.meta.get("max_dt", 0.01)
    t0 = time.perf_counter()
    s.step(max_dt)
    one = time.perf_counter() - t0
    ticks = max(1, min(200, int(budget_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(ticks):
        s.step(max_dt)
    dt = time.perf_counter() - t0
    out = {"value": tile.cells * ticks / dt, "unit": "cell-updates/s", "cores": threads,
           "kind": "port",
           "sample": f"{ticks} ticks of the {tile.nx}x{tile.ny} tile (after 1 untimed), FP64 "
                     f"reference CPU tick restated in oracle/, {threads} threads"}
    # Beside it, bounded samples of the same tick on one thread, and of the FP32 restatement of
    # the card's step (the oracle the GPU tick is held to) on one core.
    one = oracle.Solver64(g, 1)
    one.set_state(tile.h, tile.hu, tile.hv)
    one.set_inputs(tile.bed, None, tile.source)
    t0, n1 = time.perf_counter(), 0
    while time.perf_counter() - t0 < budget_s / 4 and n1 < 50:
        one.step(max_dt)
        n1 += 1
    out["one_thread"] = {"value": tile.cells * n1 / (time.perf_counter() - t0),
                         "unit": "cell-updates/s", "ticks": n1}
    r = oracle.RefStep(oracle.Grid(tile.nx, tile.ny, tile.cell_m))
    r.set_bed(tile.bed)
    if tile.source is not None:
        r.set_source(tile.source)
    r.write_state(tile.h, tile.hu, tile.hv)
    t0, n2 = time.perf_counter(), 0
    while time.perf_counter() - t0 < budget_s / 4 and n2 < 50:
        r.run_steps(1, max_dt)
        n2 += 1
    out["fp32_oracle_one_core"] = {"value": tile.cells * n2 / (time.perf_counter() - t0),
                                   "unit": "cell-updates/s", "ticks": n2}
    return out


def workload_config(tile, ticks: int, world: int) -> dict:
    """The `config` both arms print for a plain-tick workload."""
    per_tick = tile.cells * (32.125 if tile.source is not None else 28.125)
    return {
        "workload": f"plain tick {tile.nx}x{tile.ny} from the same seeded initial state, closed "
                    f"edges, max_dt {tile.meta.get('max_dt', 0.01)} s"
                    + (", rain" if tile.source is not None else ""),
        "cells": tile.cells, "ticks_per_step": ticks, "max_dt": tile.meta.get("max_dt", 0.01),
        "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
        "l2": f"{per_tick / 1e6:.1f} MB of planes a tick "
              f"({'larger' if per_tick > 129e6 else 'smaller'} than the 129 MB L2); a 512 MB "
              "write flushes L2 between steps, outside the timed events",
    }


def run_reference(args, tile, rank, world):
    """--impl reference: the reference CPU tick on this host's cores, on rank 0 only."""
    if rank != 0:
        return None
    import oracle
    threads = os.cpu_count() or 1
    g = oracle.Grid(tile.nx, tile.ny, tile.cell_m)
    s = oracle.Solver64(g, threads)
    s.set_state(tile.h, tile.hu, tile.hv)
    s.set_inputs(tile.bed, None, tile.source)
    max_dt = tile.meta.get("max_dt", 0.01)
    # The same ticks a step as the GPU arm, from the same initial state every step.
    ticks_per_step = tile.meta["ticks"]
    for _ in range(args.warmup):
        for _ in range(ticks_per_step):
            s.step(max_dt)
    dt = 0.0
    for _ in range(args.steps):
        s.set_state(tile.h, tile.hu, tile.hv)  # untimed, like the GPU arm's restore
        t0 = time.perf_counter()
        for _ in range(ticks_per_step):
            s.step(max_dt)
        dt += time.perf_counter() - t0
    value = tile.cells * ticks_per_step * args.steps / dt
    sample = (f"{ticks_per_step} ticks a step of the {tile.nx}x{tile.ny} tile, FP64 reference "
              f"CPU tick (oracle/ restatement, byte-equal to the reference's build), {threads} "
              "threads")
    return {
        "impl": "reference", "metric": "water cell-updates/s", "value": value,
        "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": tile.meta.get("data", "synthetic"),
        "config": dict(workload_config(tile, ticks_per_step, world),
                       parallelism="the host's cores, rank 0"),
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------------------------------------
# our arm

def run_plain(args, tile, rank, world):
    import torch
    from game_engine_gb300 import lib, water_live as wl

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    L = lib()
    step = wl.DeviceStep()
    cfg = wl.Config(tile.nx, tile.ny, tile.cell_m, device=dev)
    assert step.create(cfg), step.error
    ticks = tile.meta["ticks"]
    max_dt = tile.meta["max_dt"]
    n = tile.cells
    assert step.set_bed(tile.bed, 0.0), step.error
    if tile.source is not None:
        assert step.set_source(tile.source), step.error
    assert step.write_state(tile.h, tile.hu, tile.hv), step.error
    # The initial state as float planes on the device, restored before every step.
    init = torch.from_numpy(step.read_state_bits()).to(f"cuda:{dev}")
    s_ptr = step.stream()
    stream = torch.cuda.ExternalStream(s_ptr)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")

    def one_step():
        rc = L.wl_write_state_device(step.handle, C.c_void_p(init.data_ptr()), s_ptr)
        assert rc == 0, rc
        assert step.record(s_ptr, ticks, max_dt), step.error

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.add_(1.0)

    for _ in range(args.warmup):
        one_step()
        flush_l2()
    torch.cuda.synchronize(dev)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    tick_launches0 = step.tick_launches()
    with Clocks(dev) as clocks:
        for k in range(args.steps):
            starts[k].record(stream)
            one_step()
            ends[k].record(stream)
            flush_l2()
        torch.cuda.synchronize(dev)
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    tick_launches = step.tick_launches() - tick_launches0
    # Untimed: the last step's state against the oracle's hash of the same ticks.
    gold = golden_config(tile.meta.get("name"))
    oracle_equal = None
    if gold is not None and gold.get("ticks") == ticks and gold.get("max_dt") == max_dt:
        oracle_equal = step.state_hash() == gold["hash"]
        assert oracle_equal, "the timed run's state differs from the oracle's (state hash)"
    from game_engine_gb300.shard import max_over_ranks
    ms = max_over_ranks(ms)  # the slowest rank's time (gloo or NCCL group under torchrun)
    # A step: the restore and the prime, then the ticks (one resident launch for a small tile).
    launches = args.steps * 2 + tick_launches

    # The dominant kernel's average launch, from the same events: every launch of a step but two
    # (the restore and the prime, a few microseconds) is a tick, enqueued ahead of the device, so
    # a step's time over its ticks is the tick's duration with the gap between launches included
    # (a small tile's resident launch: its ticks' share of the launch, bytes and time alike).
    tick_ms = ms / args.steps / ticks
    bytes_per_cell = 28.0 + (4.0 if tile.source is not None else 0.0) + 32.0 / 256.0
    algo_bytes = bytes_per_cell * n
    achieved = algo_bytes / (tick_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "tick_traffic.json")
    if os.path.exists(tpath):
        try:
            with open(tpath) as f:
                tr = json.load(f)
            traffic = tr.get(tile.meta.get("name"))
        except Exception:
            traffic = None
    ledger = step.read_ledger()

    # e2e: the public C ABI with host buffers (pinned), every step uploads and reads back.
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).pin_memory()
    h_h, h_hu, h_hv, h_bed = pin(tile.h), pin(tile.hu), pin(tile.hv), pin(tile.bed)
    h_src = pin(tile.source) if tile.source is not None else None
    o_h = torch.empty(n, dtype=torch.float64).pin_memory()
    o_hu = torch.empty(n, dtype=torch.float64).pin_memory()
    o_hv = torch.empty(n, dtype=torch.float64).pin_memory()
    dp = C.POINTER(C.c_double)
    ptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), dp)
    err = C.create_string_buffer(256)

    def e2e_step():
        assert L.wl_set_bed(step.handle, ptr(h_bed), n, 0.0, err, 256) == 0, err.value
        if h_src is not None:
            assert L.wl_set_source(step.handle, ptr(h_src), n, 1, 0, err, 256) == 0, err.value
        assert L.wl_write_state(step.handle, ptr(h_h), ptr(h_hu), ptr(h_hv), n, err, 256) == 0
        assert L.wl_run_steps(step.handle, ticks, max_dt, err, 256) == 0, err.value
        assert L.wl_read_state(step.handle, ptr(o_h), ptr(o_hu), ptr(o_hv), n, err, 256) == 0

    for _ in range(max(1, args.warmup)):
        e2e_step()
    e2e_s = 0.0
    for _ in range(args.steps):
        flush_l2()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e2e_step()
        e2e_s += time.perf_counter() - t0
    h2d = n * 8 * (4 + (1 if h_src is not None else 0))
    d2h = n * 8 * 3

    total_cells = n * ticks * args.steps * world
    value = total_cells / (ms * 1e-3)
    e2e_value = total_cells / e2e_s
    out = {
        "metric": "water cell-updates/s", "value": value, "unit": "cell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": tile.meta.get("data", "synthetic"),
        "config": workload_config(tile, ticks, world),
        "ledger_steps_last_run": ledger["steps"] if ledger else None,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "algorithmic_bytes_per_launch": algo_bytes,
                     "bytes_per_cell": bytes_per_cell, "avg_launch_ms": tick_ms,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "state_hash_equals_oracle": oracle_equal,
    }
    return out


def run_tiles(steps: int, warmup: int, ticks: int = 0, count: int = 4096):
    """The batched configuration: `count` tiles of seeded uneven sides, `ticks` ticks a step, one
    persistent CUDA-graph-captured launch a tick after the autotuner's choice; beside it the
    per-tile-launch form (one launch per tile per tick) on the same tiles, its best of five
    launch forms."""
    import torch
    from game_engine_gb300 import workloads
    from game_engine_gb300.batch import Batch, concat

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ticks = ticks or 200
    tiles = workloads.tiles_4096(count)
    sides = [(t.nx, t.ny) for t in tiles]
    b = Batch(sides, device=dev)
    b.set_bed(concat(tiles, "bed"))
    h0 = concat(tiles, "h")
    b.write_state(h0)
    cells = b.cells
    del tiles
    tuning = b.autotune(workloads.MAX_DT, trial_ticks=4)
    stream = torch.cuda.ExternalStream(b.stream())
    for _ in range(warmup):
        b.run_ticks(ticks // 4, workloads.MAX_DT)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ms = 0.0
    for _ in range(steps):
        b.write_state(h0)  # the same initial state every step (untimed)
        ev[0].record(stream)
        b.run_ticks(ticks, workloads.MAX_DT, graph=True)
        ev[1].record(stream)
        torch.cuda.synchronize(dev)
        ms += ev[0].elapsed_time(ev[1])
    batched = cells * ticks * steps / (ms * 1e-3)
    # Untimed: every tile's state after the last step's ticks against the oracle's hashes.
    gold = golden_config("tiles_4096")
    hashes_equal = None
    if gold is not None and gold["count"] == count and gold["ticks"] == ticks:
        got = [int(h) for h in b.tile_hashes()]
        hashes_equal = got == gold["hashes"]
        assert hashes_equal, (f"{sum(a != w for a, w in zip(got, gold['hashes']))} of {count} "
                              "tiles differ from the oracle's hashes")
    # The per-tile-launch form on the same tiles, timed five ways: 16-row marches on one stream,
    # from a captured graph, and dealt to 64 concurrent streams as independent steps would run;
    # and the three-phase blocks (the small-tile shape) on 64 streams, with their loads and staged
    # by tensor copies. The best of them is the comparison. Fewer ticks: it is slow.
    per_ticks = 10
    per = {}
    for name, graph, nstreams, rows, stage in (
            ("stream", False, 1, 16, 0), ("graph", True, 1, 16, 0),
            ("streams_64", False, 64, 16, 0), ("streams_64_blocks", False, 64, 1, 0),
            ("streams_64_blocks_staged", False, 64, 1, 1)):
        b.set_tuning(rows, 0, stage=stage)
        b.write_state(h0)
        b.run_tile_ticks(2, workloads.MAX_DT, graph=graph, streams=nstreams)
        ev[0].record(stream)
        b.run_tile_ticks(per_ticks, workloads.MAX_DT, graph=graph, streams=nstreams)
        ev[1].record(stream)
        torch.cuda.synchronize(dev)
        per[name] = cells * per_ticks / (ev[0].elapsed_time(ev[1]) * 1e-3)
    per_tile = max(per.values())
    b.close()
    return {
        "workload": f"{count} tiles, sides from {workloads.TILE_SIDES}, own fBm 0-20 m and a 2 m "
                    f"column each, {ticks} ticks a step, max_dt 0.01 s",
        "cells": cells, "tiles": count, "value": batched, "unit": "cell-updates/s",
        "ms_per_tick": ms / (steps * ticks), "tuning": tuning,
        "per_tile_launch": {"value": per_tile, "unit": "cell-updates/s", "forms": per,
                            "best": max(per, key=per.get)},
        "speedup_vs_per_tile_launch": batched / per_tile,
        "tile_hashes_equal_oracle": hashes_equal,
        "launches_per_tick": {"batched": 1, "per_tile": count},
    }


def _time_on(stream, fn, steps):
    """Milliseconds of `steps` calls of fn, CUDA events on `stream` around each."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for a, b in ev:
        a.record(stream)
        fn()
        b.record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def run_adjoint(steps: int, warmup: int, ticks: int = 0):
    """The adjoint configuration (512 x 512, 2000 ticks, a checkpoint every 50, 64 probes): the
    whole sweep (checkpoint pass, loss, recompute and reverse ticks) from one captured graph, in
    seconds per tick, against the plain tick's own seconds per tick on the same tile."""
    import torch
    from game_engine_gb300 import lib, water_live as wl, workloads
    from game_engine_gb300.adjoint import Adjoint

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    t = workloads.adjoint_512()
    ticks, every, dt = ticks or t.meta["ticks"], t.meta["every"], t.meta["max_dt"]
    probes = t.meta["probes"]

    def make(bed):
        s = wl.DeviceStep()
        assert s.create(wl.Config(t.nx, t.ny, t.cell_m, device=dev)), s.error
        assert s.set_bed(bed) and s.set_source(t.source) and s.write_state(t.h, t.hu, t.hv)
        return s

    # The targets: the plain tick on the bed plus N(0, 0.1 m).
    tgt = make(workloads.perturbed_bed(t.bed, workloads.SEEDS["adjoint_512"]))
    assert tgt.run_steps(ticks, dt), tgt.error
    targets = tgt.read_state()[0][probes]
    tgt.destroy()
    step = make(t.bed)
    a = Adjoint(step, ticks, every, probes, targets)
    s_ptr = step.stream()
    stream = torch.cuda.ExternalStream(s_ptr)
    for _ in range(warmup):
        a.run(dt)
    sweep_ms = _time_on(stream, lambda: a.run(dt), steps)
    loss, g_bed, g_src, limited = a.read()
    launches = a.launches()
    nbytes = a.device_bytes()
    a.close()
    # The plain tick's cost on the same tile: the same ticks from the same state.
    init = torch.from_numpy(step.read_state_bits()).to(f"cuda:{dev}")
    L = lib()

    def forward():
        assert L.wl_write_state_device(step.handle, C.c_void_p(init.data_ptr()), s_ptr) == 0
        assert step.record(s_ptr, ticks, dt), step.error

    for _ in range(warmup):
        forward()
    fwd_ms = _time_on(stream, forward, steps)
    step.destroy()
    sweep_tick = statistics.median(sweep_ms) * 1e-3 / ticks
    fwd_tick = statistics.median(fwd_ms) * 1e-3 / ticks
    return {
        "workload": f"adjoint_512: {t.nx} x {t.ny}, {ticks} ticks of {dt} s, a checkpoint every "
                    f"{every}, {len(probes)} probes, the source on at zero inflow, targets from a "
                    f"run on the bed + N(0, 0.1 m)",
        "metric": "fwd+adjoint s/tick", "value": sweep_tick, "unit": "s/tick",
        "forward_s_per_tick": fwd_tick, "ratio_to_forward": sweep_tick / fwd_tick,
        "loss": float(loss[0]), "shortened_ticks": int(limited[0]),
        "gpu_launches_per_sweep": launches, "device_bytes": nbytes,
        "grad_norms": {"bed": float(np.abs(g_bed).max()), "source": float(np.abs(g_src).max())},
    }


def run_tick_queue(steps: int, warmup: int, sides=(256, 2048), frame_slots: int = 16):
    """The tick queue (water_live.md:76-94): ticks of 1/60 s queued on the device and stepped by
    a captured graph of `frame_slots` slots (one frame's worth). Per tile side: microseconds a
    busy slot (every slot steps), the plain tick's microseconds on the same tile and state, and
    microseconds an idle slot (nothing queued)."""
    import torch
    from game_engine_gb300 import water_live as wl, workloads
    from game_engine_gb300.tick_queue import TickQueue

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    tick = float(np.float32(1.0 / 60.0))
    out = {"metric": "slot time", "unit": "us", "frame_slots": frame_slots,
           "launches_per_slot": TickQueue.launches_per_slot(), "tiles": {}}
    for side in sides:
        t = workloads.plain_256() if side == 256 else workloads.plain_2048(side)

        def make():
            st = wl.DeviceStep()
            assert st.create(wl.Config(t.nx, t.ny, t.cell_m, device=dev)), st.error
            assert st.set_bed(t.bed) and st.write_state(t.h, t.hu, t.hv), st.error
            if t.source is not None:
                assert st.set_source(t.source), st.error
            return st

        # The plain tick on the same state: free-running sub-steps of the stable length.
        plain = make()
        s_ptr = plain.stream()
        stream = torch.cuda.ExternalStream(s_ptr)
        for _ in range(warmup):
            assert plain.record(s_ptr, frame_slots, float("inf")), plain.error
        plain_ms = _time_on(stream, lambda: plain.record(s_ptr, frame_slots, float("inf")), steps)
        plain.destroy()

        step = make()
        q = TickQueue(step, records=64)
        g_stream = torch.cuda.Stream(device=dev)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=g_stream):
            assert q.enqueue_slots(torch.cuda.current_stream().cuda_stream, frame_slots)

        def frame():  # a replay on the stream the events are recorded on
            with torch.cuda.stream(g_stream):
                graph.replay()

        busy, n_tick = [], 0
        for k in range(warmup + steps):
            # 3 frames of ticks queued (a sub-step or more each), one frame's slots timed.
            while q.status()["pushed"] - q.status()["landed"] < 3 * frame_slots:
                assert q.push(n_tick, tick), q.error
                n_tick += 1
            before = int(step.read_ledger_bits()[10])  # the ledger's step count
            ms = _time_on(g_stream, frame, 1)[0]
            assert int(step.read_ledger_bits()[10]) - before == frame_slots  # every slot stepped
            if k >= warmup:
                busy.append(ms)
        for _ in range(100000):  # drain
            st = q.status()
            if st["landed"] == st["pushed"]:
                break
            frame()
            torch.cuda.synchronize()
        idle = _time_on(g_stream, frame, steps)
        landed = q.status()["landed"]
        subs = [r["substeps"] for r in q.landed(max(0, landed - 16), min(16, landed))]
        q.close()
        step.destroy()
        busy_us = statistics.median(busy) * 1e3 / frame_slots
        plain_us = statistics.median(plain_ms) * 1e3 / frame_slots
        out["tiles"][f"{t.nx}x{t.ny}"] = {
            "busy_slot_us": busy_us, "plain_tick_us": plain_us,
            "overhead_us": busy_us - plain_us, "idle_slot_us": statistics.median(idle) * 1e3 /
            frame_slots, "cell_updates_per_s": t.cells / (busy_us * 1e-6),
            "substeps_per_tick": subs, "ticks_landed": landed}
    return out


def run_full_step(steps: int, warmup: int, side: int = 2048, ticks: int = 20, cpu_budget_s=10.0):
    """The complete FP64 step (water_state::Solver with every input) on the device: seconds a step
    and cell-updates/s over `ticks` steps of max_dt 0.01 from the same state, against the oracle's
    restatement of the reference's CPU step on one host core, a bounded sample of steps."""
    import torch
    from game_engine_gb300 import water_state as ws, workloads
    dev_index = int(os.environ.get("LOCAL_RANK", "0"))
    t, config, fields, inputs = workloads.full_step(side)
    s = ws.Solver(ws.Config(config["nx"], config["ny"], config["cell_m"], carried=config["carried"],
                            device=dev_index))
    for name, v in fields.items():
        s.set(name, v)
    s.set_inputs(inputs)
    stream = torch.cuda.ExternalStream(s.stream())
    snapshot = {name: s.get(name) for name in fields}

    def run():
        assert s.enqueue_steps(s.stream(), ticks, 0.01)

    for _ in range(warmup):
        run()
    torch.cuda.synchronize()
    ms = _time_on(stream, run, steps)
    launches = ticks * 6 + 1
    device_bytes = s.device_bytes()
    s.close()
    step_s = statistics.median(ms) * 1e-3 / ticks
    out = {"workload": f"the complete FP64 step, {t.nx}x{t.ny}: {t.meta['data']}; Manning 0.03, "
                       "a ground store, a foam and a sediment; max_dt 0.01 s",
           "metric": "cell-updates/s", "value": t.cells / step_s, "unit": "cell-updates/s",
           "s_per_step": step_s, "steps_per_run": ticks, "gpu_launches_per_run": launches,
           "device_bytes": device_bytes, "dtype": "f64"}
    try:
        import oracle
        o = oracle.FullSolver(config["nx"], config["ny"], config["cell_m"],
                              carried=config["carried"])
        for name, v in snapshot.items():
            o.set(name, v)
        o.step(inputs, 0.01)  # untimed
        n_cpu, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < cpu_budget_s and n_cpu < ticks:
            o.step(inputs, 0.01)
            n_cpu += 1
        cpu_s = (time.perf_counter() - t0) / max(n_cpu, 1)
        out["cpu_baseline"] = {"value": t.cells / cpu_s, "unit": "cell-updates/s", "cores": 1,
                               "kind": "port",
                               "sample": f"{n_cpu} steps of the same tile (after 1 untimed), the "
                                         "reference's complete FP64 step restated in oracle/, one "
                                         "thread"}
    except Exception as e:  # the oracle is test infrastructure; the number is reported if it runs
        out["cpu_baseline"] = {"unavailable": str(e)[:200]}
    return out


def run_tiles_adjoint(steps: int, warmup: int, ticks: int = 0, count: int = 256):
    """The batched adjoint configuration (256 tiles, 500 ticks, a checkpoint every 25, 64 probes
    a tile): the sweep over every tile in one launch a tick forward and reverse, from one captured
    graph, against the batched plain tick on the same tiles."""
    import torch
    from game_engine_gb300 import workloads
    from game_engine_gb300.adjoint import Adjoint
    from game_engine_gb300.batch import Batch, concat

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    tiles = workloads.tiles_256_adjoint(count)
    ticks, every, dt = (ticks or workloads.TILES_ADJOINT_TICKS, workloads.TILES_ADJOINT_EVERY,
                        workloads.MAX_DT)
    sides = [(t.nx, t.ny) for t in tiles]
    seed = workloads.SEEDS["tiles_256_adjoint"]

    def make(beds):
        b = Batch(sides, device=dev)
        b.set_bed(np.concatenate(beds))
        b.set_source(concat(tiles, "source"))
        b.write_state(concat(tiles, "h"))
        return b

    tgt = make([workloads.perturbed_bed(t.bed, seed + k) for k, t in enumerate(tiles)])
    tgt.run_ticks(ticks, dt)
    targets = [tgt.read_tile_bits(k)[:t.cells][t.meta["probes"]].astype(np.float64)
               for k, t in enumerate(tiles)]
    tgt.close()
    b = make([t.bed for t in tiles])
    b.autotune(dt, trial_ticks=3)
    a = Adjoint(b, ticks, every, [t.meta["probes"] for t in tiles], targets)
    stream = torch.cuda.ExternalStream(b.stream())
    for _ in range(warmup):
        a.run(dt)
    sweep_ms = _time_on(stream, lambda: a.run(dt), steps)
    loss, _, _, limited = a.read()
    launches = a.launches()
    nbytes = a.device_bytes()
    a.close()
    h0 = concat(tiles, "h")

    def forward():
        b.write_state(h0)
        b.run_ticks(ticks, dt, graph=True)

    forward()
    fwd_ms = _time_on(stream, lambda: b.run_ticks(ticks, dt, graph=True), steps)
    cells = b.cells
    b.close()
    sweep_tick = statistics.median(sweep_ms) * 1e-3 / ticks
    fwd_tick = statistics.median(fwd_ms) * 1e-3 / ticks
    return {
        "workload": f"tiles_256_adjoint: {count} tiles, sides from "
                    f"{workloads.ADJOINT_TILE_SIDES}, {cells} cells, {ticks} ticks of {dt} s, "
                    f"a checkpoint every {every}, 64 probes a tile",
        "metric": "fwd+adjoint s/tick", "value": sweep_tick, "unit": "s/tick",
        "forward_s_per_tick": fwd_tick, "ratio_to_forward": sweep_tick / fwd_tick,
        "loss_sum": float(loss.sum()), "shortened_ticks": int(limited.sum()),
        "gpu_launches_per_sweep": launches, "device_bytes": nbytes,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plain_2048")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched and adjoint measurements beside the headline")
    ap.add_argument("--tiles", type=int, default=4096,
                    help="tiles of the batched workload (a smaller batch for a profiler; the "
                         "configuration's number is measured with the default)")
    ap.add_argument("--ticks", type=int, default=0,
                    help="ticks a step instead of the workload's (a short run for a profiler; "
                         "the configuration's number is measured with the default)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    from game_engine_gb300 import workloads

    if args.workload == "tick_queue":
        if rank == 0:
            print(json.dumps(run_tick_queue(args.steps, args.warmup)), flush=True)
        return
    if args.workload == "full_step":
        if rank == 0:
            print(json.dumps(run_full_step(args.steps, args.warmup)), flush=True)
        return
    if args.workload in ("tiles_4096", "adjoint_512", "tiles_256_adjoint"):
        if rank == 0:
            fn = {"tiles_4096": run_tiles, "adjoint_512": run_adjoint,
                  "tiles_256_adjoint": run_tiles_adjoint}[args.workload]
            if args.workload == "tiles_4096":
                out = run_tiles(args.steps, args.warmup, args.ticks, count=args.tiles)
            else:
                out = fn(args.steps, args.warmup, args.ticks)
            print(json.dumps(out), flush=True)
        return
    # The reference arm builds its terrain with the numpy generator (the same doubles), so that
    # nothing of this library is loaded into its process.
    terrain = workloads.fbm_numpy if args.impl == "reference" else workloads.fbm
    if args.workload == "plain_2048":
        tile = workloads.plain_2048(terrain=terrain)
    elif args.workload == "plain_256":
        tile = workloads.plain_256(terrain=terrain)
    elif args.workload == "plain_1024":
        # The throughput tile's terrain, depth and rain at 1024 x 1024: a tile of the three-phase
        # block shape in 256-thread CTAs (2048 blocks), the staged block tick's, for a profiler.
        tile = workloads.plain_2048(1024, terrain=terrain)
    else:
        raise SystemExit(f"unknown workload {args.workload}")
    if args.ticks > 0:
        tile.meta["ticks"] = args.ticks

    if args.impl == "reference":
        out = run_reference(args, tile, rank, world)
        if out is not None:
            print(json.dumps(out), flush=True)
        return

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("WL_BENCH_NCCL") else "gloo")
    out = run_plain(args, tile, rank, world)
    if rank == 0 and not args.no_extras:
        out["batched"] = run_tiles(max(1, min(args.steps, 3)), 1)
        out["adjoint"] = run_adjoint(max(1, min(args.steps, 3)), 1)
        out["batched_adjoint"] = run_tiles_adjoint(max(1, min(args.steps, 3)), 1)
        out["tick_queue"] = run_tick_queue(max(3, min(args.steps, 10)), 3)
        out["full_step"] = run_full_step(max(3, min(args.steps, 5)), 1,
                                         cpu_budget_s=0.0 if args.no_cpu else 10.0)
    if rank == 0:
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline(tile, os.cpu_count() or 1)
        else:
            out["cpu_baseline"] = None
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()

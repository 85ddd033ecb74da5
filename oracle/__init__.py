"""ORACLE — test infrastructure only.

ctypes bindings over the CPU restatement (``oracle/_build/liboracle.so``, built by
``oracle/Makefile``) and, where it was built, over the reference's own compiled CPU solver
(``oracle/_ref/libwsref.so``, built by ``oracle/build_ref.sh`` from the reference's sources).
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this
package, always as the checker or the CPU baseline, never as the thing measured or shipped.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libwsref.so")

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_lib = None
_ref = None


def build(quiet: bool = True) -> None:
    """Compiles the restatement (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


def build_ref(reference_root: str | None = None) -> bool:
    """Compiles the reference's own solver when its sources are present; True if built. The root
    is `reference_root`, else $WL_REFERENCE_ROOT, else the recipe's own (oracle/build_ref.sh)."""
    cmd = [os.path.join(HERE, "build_ref.sh")]
    if reference_root:
        cmd.append(reference_root)
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
    return os.path.exists(REF_PATH)


def reference_root() -> str | None:
    """The reference's source root: $WL_REFERENCE_ROOT, else the root oracle/_ref was built from
    (recorded by oracle/build_ref.sh); None when neither names a directory that exists."""
    root = os.environ.get("WL_REFERENCE_ROOT")
    if not root:
        try:
            with open(os.path.join(HERE, "_ref", "reference_root")) as f:
                root = f.read().strip()
        except OSError:
            return None
    return root if root and os.path.isdir(root) else None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.oracle_hash_floats.restype = C.c_uint64
        L.oracle_hash_floats.argtypes = [_fp, C.c_size_t]
        L.oracle_step_create.restype = C.c_void_p
        L.oracle_step_create.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double,
                                         C.c_double, C.c_double, C.c_uint32, C.c_int, C.c_int]
        for name, args in [
            ("oracle_step_destroy", [C.c_void_p]),
            ("oracle_step_write_state", [C.c_void_p, _dp, _dp, _dp]),
            ("oracle_step_set_bed", [C.c_void_p, _dp, C.c_double]),
            ("oracle_step_set_manning", [C.c_void_p, _dp]),
            ("oracle_step_set_source", [C.c_void_p, _dp, C.c_uint32, C.c_int]),
            ("oracle_step_run_steps", [C.c_void_p, C.c_uint32, C.c_double]),
            ("oracle_step_run_length_pass", [C.c_void_p, C.c_double]),
            ("oracle_step_prime", [C.c_void_p]),
            ("oracle_step_read_ledger", [C.c_void_p, _dp]),
            ("oracle_step_read_state_f32", [C.c_void_p, _fp]),
            ("oracle_step_read_state_f64", [C.c_void_p, _dp]),
            ("oracle_step_write_planes_f32", [C.c_void_p, _fp]),
            ("oracle_step_read_partials", [C.c_void_p, _fp]),
            ("oracle_step_read_ledger_bits", [C.c_void_p, C.c_void_p]),
        ]:
            f = getattr(L, name)
            f.restype = None
            f.argtypes = args
        L.oracle_step_advance.restype = C.c_uint64
        L.oracle_step_advance.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_int)]
        L.oracle_step_state_hash.restype = C.c_uint64
        L.oracle_step_state_hash.argtypes = [C.c_void_p]
        L.oracle_step_group_count.restype = C.c_uint32
        L.oracle_step_group_count.argtypes = [C.c_void_p]
        L.oracle_solver_create.restype = C.c_void_p
        L.oracle_solver_create.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double,
                                           C.c_double, C.c_double, C.c_uint32, C.c_uint32]
        for name, args in [
            ("oracle_solver_destroy", [C.c_void_p]),
            ("oracle_solver_set_state", [C.c_void_p, _dp, _dp, _dp]),
            ("oracle_solver_set_inputs", [C.c_void_p, _dp, _dp, _dp]),
            ("oracle_solver_get_state", [C.c_void_p, _dp, _dp, _dp]),
            ("oracle_solver_ledger", [C.c_void_p, _dp]),
        ]:
            f = getattr(L, name)
            f.restype = None
            f.argtypes = args
        L.oracle_solver_step.restype = C.c_double
        L.oracle_solver_step.argtypes = [C.c_void_p, C.c_double]
        L.oracle_solver_advance.restype = C.c_uint64
        L.oracle_solver_advance.argtypes = [C.c_void_p, C.c_double]
        L.oracle_solver_state_hash.restype = C.c_uint64
        L.oracle_solver_state_hash.argtypes = [C.c_void_p]
        L.oracle_solver_volume.restype = C.c_double
        L.oracle_solver_volume.argtypes = [C.c_void_p]
        _u32p = C.POINTER(C.c_uint32)
        grid_args = [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_double,
                     C.c_uint32]
        L.oracle_adj_forward.restype = C.c_uint32
        L.oracle_adj_forward.argtypes = grid_args + [C.c_int, C.c_double, C.c_uint32, _dp, _dp,
                                                     _dp, _dp]
        L.oracle_adjoint.restype = C.c_uint32
        L.oracle_adjoint.argtypes = grid_args + [C.c_int, C.c_double, C.c_uint32, _dp, _dp, _dp,
                                                 _u32p, _dp, C.c_uint32, _dp, _dp, _dp, _dp]
        L.oracle_adjoint_mixed.restype = C.c_uint32
        L.oracle_adjoint_mixed.argtypes = grid_args + [C.c_double, C.c_uint32, _dp, _dp, _dp,
                                                       _u32p, _dp, C.c_uint32, _dp, _dp, _dp]
        L.oracle_adj_fd.restype = None
        L.oracle_adj_fd.argtypes = grid_args + [C.c_double, C.c_uint32, _dp, _dp, _dp, _u32p, _dp,
                                                C.c_uint32, _u32p, C.c_uint32, C.c_double,
                                                C.c_double, _dp, _dp, C.c_uint32]
        L.oracle_adj_loss64.restype = C.c_double
        L.oracle_adj_loss64.argtypes = grid_args + [C.c_double, C.c_uint32, _dp, _dp, _dp, _u32p,
                                                    _dp, C.c_uint32]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.wsref_create.restype = C.c_void_p
        R.wsref_create.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_uint32, C.c_uint32]
        for name, args in [
            ("wsref_destroy", [C.c_void_p]),
            ("wsref_set_state", [C.c_void_p, _dp, _dp, _dp]),
            ("wsref_set_inputs", [C.c_void_p, _dp, _dp, _dp]),
            ("wsref_get_state", [C.c_void_p, _dp, _dp, _dp]),
            ("wsref_ledger", [C.c_void_p, _dp]),
        ]:
            f = getattr(R, name)
            f.restype = None
            f.argtypes = args
        R.wsref_step.restype = C.c_double
        R.wsref_step.argtypes = [C.c_void_p, C.c_double]
        R.wsref_advance.restype = C.c_uint64
        R.wsref_advance.argtypes = [C.c_void_p, C.c_double]
        R.wsref_state_hash.restype = C.c_uint64
        R.wsref_state_hash.argtypes = [C.c_void_p]
        R.wsref_volume.restype = C.c_double
        R.wsref_volume.argtypes = [C.c_void_p]
        _ref = R
    return _ref


def _d(a):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.ctypes.data_as(_dp)


def _keep(*arrays):
    return [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in arrays]


@dataclass
class Grid:
    """The fields of water_state::Config the step reads (water_state.h:83-99)."""
    nx: int
    ny: int
    cell_m: float = 1.0
    gravity: float = 9.81
    cfl: float = 0.45
    dry_depth_m: float = 1e-9
    open_edges: int = 0  # bits: 1 west, 2 east, 4 south, 8 north

    @property
    def cells(self) -> int:
        return self.nx * self.ny


class RefStep:
    """The card's step on the CPU (water_step.slang + water_live.cpp's host half)."""

    def __init__(self, grid: Grid, fixed_ops: bool = False, precision64: bool = False):
        L = lib()
        self.grid = grid
        self.is64 = precision64
        self.h = L.oracle_step_create(grid.nx, grid.ny, grid.cell_m, grid.gravity, grid.cfl,
                                      grid.dry_depth_m, grid.open_edges, int(fixed_ops),
                                      int(precision64))
        if not self.h:
            raise ValueError("oracle: an empty grid")

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_step_destroy(self.h)
            self.h = None

    def write_state(self, h, hu, hv):
        h, hu, hv = _keep(h, hu, hv)
        lib().oracle_step_write_state(self.h, _d(h), _d(hu), _d(hv))

    def set_bed(self, bed, datum=0.0):
        (bed,) = _keep(bed)
        lib().oracle_step_set_bed(self.h, _d(bed), float(datum))

    def set_manning(self, m):
        (m,) = _keep(m)
        lib().oracle_step_set_manning(self.h, _d(m))

    def set_source(self, s, every=1, compensate=False):
        (s,) = _keep(s)
        lib().oracle_step_set_source(self.h, _d(s), int(every), int(compensate))

    def run_steps(self, count, max_dt):
        lib().oracle_step_run_steps(self.h, int(count), float(max_dt))

    def run_length_pass(self, max_dt):
        lib().oracle_step_run_length_pass(self.h, float(max_dt))

    def prime(self):
        """prime_main: the records of the state as it stands (slang:373-386)."""
        lib().oracle_step_prime(self.h)

    def read_ledger(self):
        out = np.zeros(6)
        lib().oracle_step_read_ledger(self.h, out.ctypes.data_as(_dp))
        return dict(source_m3=out[0], open_edge_out_m3=out[1], roundoff_m3=out[2],
                    time_s=out[3], remaining_s=out[4], steps=int(out[5]))

    def advance(self, duration):
        refused = C.c_int(0)
        steps = lib().oracle_step_advance(self.h, float(duration), C.byref(refused))
        return steps, bool(refused.value)

    def read_state_bits(self):
        n = self.grid.cells
        if self.is64:
            out = np.zeros(4 * n, dtype=np.float64)
            lib().oracle_step_read_state_f64(self.h, out.ctypes.data_as(_dp))
        else:
            out = np.zeros(4 * n, dtype=np.float32)
            lib().oracle_step_read_state_f32(self.h, out.ctypes.data_as(_fp))
        return out

    def write_planes(self, planes):
        p = np.ascontiguousarray(planes, dtype=np.float32)
        lib().oracle_step_write_planes_f32(self.h, p.ctypes.data_as(_fp))

    def state_hash(self):
        return int(lib().oracle_step_state_hash(self.h))

    def group_count(self):
        return int(lib().oracle_step_group_count(self.h))

    def read_partials_bits(self):
        out = np.zeros(8 * self.group_count(), dtype=np.float32)
        lib().oracle_step_read_partials(self.h, out.ctypes.data_as(_fp))
        return out.reshape(-1, 8)

    def read_ledger_bits(self):
        out = np.zeros(12, dtype=np.uint32)
        lib().oracle_step_read_ledger_bits(self.h, out.ctypes.data_as(C.c_void_p))
        return out


class Solver64:
    """The reference CPU tick restated (water_state.cpp): depth and momenta, FP64."""

    def __init__(self, grid: Grid, threads: int = 1):
        self.grid = grid
        self.h = lib().oracle_solver_create(grid.nx, grid.ny, grid.cell_m, grid.gravity,
                                            grid.cfl, grid.dry_depth_m, grid.open_edges,
                                            int(threads))
        self._inputs = None

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_solver_destroy(self.h)
            self.h = None

    def set_state(self, h, hu=None, hv=None):
        n = self.grid.cells
        hu = np.zeros(n) if hu is None else hu
        hv = np.zeros(n) if hv is None else hv
        h, hu, hv = _keep(h, hu, hv)
        lib().oracle_solver_set_state(self.h, _d(h), _d(hu), _d(hv))

    def set_inputs(self, bed, manning=None, source=None):
        bed, manning, source = _keep(bed, manning, source)
        lib().oracle_solver_set_inputs(self.h, _d(bed), _d(manning), _d(source))

    def step(self, max_dt):
        return lib().oracle_solver_step(self.h, float(max_dt))

    def advance(self, duration):
        return int(lib().oracle_solver_advance(self.h, float(duration)))

    def state(self):
        n = self.grid.cells
        h, hu, hv = np.zeros(n), np.zeros(n), np.zeros(n)
        lib().oracle_solver_get_state(self.h, _d(h), _d(hu), _d(hv))
        return h, hu, hv

    def state_hash(self):
        return int(lib().oracle_solver_state_hash(self.h))

    def ledger(self):
        out = np.zeros(5)
        lib().oracle_solver_ledger(self.h, out.ctypes.data_as(_dp))
        return dict(source_m3=out[0], open_edge_out_m3=out[1], roundoff_m3=out[2],
                    time_s=out[3], steps=int(out[4]))

    def volume(self):
        return lib().oracle_solver_volume(self.h)


class RefSolver:
    """The reference's own compiled water_state::Solver (oracle/_ref), where it was built."""

    def __init__(self, grid: Grid, workers: int = 0):
        R = ref()
        self.grid = grid
        self.h = R.wsref_create(grid.nx, grid.ny, grid.cell_m, grid.gravity, grid.cfl,
                                grid.dry_depth_m, grid.open_edges, int(workers))

    def __del__(self):
        if getattr(self, "h", None):
            ref().wsref_destroy(self.h)
            self.h = None

    def set_state(self, h, hu=None, hv=None):
        n = self.grid.cells
        hu = np.zeros(n) if hu is None else hu
        hv = np.zeros(n) if hv is None else hv
        h, hu, hv = _keep(h, hu, hv)
        ref().wsref_set_state(self.h, _d(h), _d(hu), _d(hv))

    def set_inputs(self, bed, manning=None, source=None):
        bed, manning, source = _keep(bed, manning, source)
        self._inputs = (bed, manning, source)
        ref().wsref_set_inputs(self.h, _d(bed), _d(manning), _d(source))

    def step(self, max_dt):
        return ref().wsref_step(self.h, float(max_dt))

    def advance(self, duration):
        return int(ref().wsref_advance(self.h, float(duration)))

    def state(self):
        n = self.grid.cells
        h, hu, hv = np.zeros(n), np.zeros(n), np.zeros(n)
        ref().wsref_get_state(self.h, _d(h), _d(hu), _d(hv))
        return h, hu, hv

    def state_hash(self):
        return int(ref().wsref_state_hash(self.h))

    def ledger(self):
        out = np.zeros(5)
        ref().wsref_ledger(self.h, out.ctypes.data_as(_dp))
        return dict(source_m3=out[0], open_edge_out_m3=out[1], roundoff_m3=out[2],
                    time_s=out[3], steps=int(out[4]))

    def volume(self):
        return ref().wsref_volume(self.h)


# ---- the adjoint's checks --------------------------------------------------------------------

def _grid_args(grid: Grid):
    return (grid.nx, grid.ny, grid.cell_m, grid.gravity, grid.cfl, grid.dry_depth_m,
            grid.open_edges)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def adj_forward(grid: Grid, dt, ticks, bed, source, state0, precision64=False):
    """`ticks` ticks of fixed length `dt` (the adjoint's forward: native ops, no Manning, no
    compensation, the source every step) from `state0` (3 planes: h, hu, hv). Returns the final
    state (3, n) and the number of ticks the card would have shortened."""
    bed, source, state0 = _keep(bed, source, state0)
    out = np.zeros(3 * grid.cells)
    lim = lib().oracle_adj_forward(*_grid_args(grid), int(precision64), float(dt), int(ticks),
                                   _d(bed), _d(source), _d(state0), _d(out))
    return out.reshape(3, -1), int(lim)


def adjoint(grid: Grid, dt, ticks, bed, source, state0, probes, targets, precision64=True,
            state_gradient=False):
    """The loss sum_p (h_T(p) - target_p)^2 and its gradients with respect to the bed and the
    source by the reverse sweep. Returns (loss, g_bed, g_source, shortened ticks), and with
    state_gradient the gradient with respect to the starting state (3 planes) after them."""
    bed, source, state0, targets = _keep(bed, source, state0, targets)
    probes = _u32(probes)
    g_bed = np.zeros(grid.cells)
    g_src = np.zeros(grid.cells)
    g_u0 = np.zeros(3 * grid.cells) if state_gradient else None
    loss = C.c_double(0.0)
    lim = lib().oracle_adjoint(*_grid_args(grid), int(precision64), float(dt), int(ticks),
                               _d(bed), _d(source), _d(state0),
                               probes.ctypes.data_as(C.POINTER(C.c_uint32)), _d(targets),
                               probes.size, C.byref(loss), _d(g_bed), _d(g_src), _d(g_u0))
    if state_gradient:
        return loss.value, g_bed, g_src, int(lim), g_u0
    return loss.value, g_bed, g_src, int(lim)


def adjoint_mixed(grid: Grid, dt, ticks, bed, source, state0, probes, targets):
    """The FP32 forward with the FP64 reverse sweep over it: (loss, g_bed, g_source, shortened)."""
    bed, source, state0, targets = _keep(bed, source, state0, targets)
    probes = _u32(probes)
    g_bed = np.zeros(grid.cells)
    g_src = np.zeros(grid.cells)
    loss = C.c_double(0.0)
    lim = lib().oracle_adjoint_mixed(*_grid_args(grid), float(dt), int(ticks), _d(bed),
                                     _d(source), _d(state0),
                                     probes.ctypes.data_as(C.POINTER(C.c_uint32)), _d(targets),
                                     probes.size, C.byref(loss), _d(g_bed), _d(g_src))
    return loss.value, g_bed, g_src, int(lim)


def adj_fd(grid: Grid, dt, ticks, bed, source, state0, probes, targets, cells, eps_bed=1e-3,
           rel_source=1e-3, threads=0, with_source=True):
    """Central differences of the FP64 replay's loss at `cells`: on the bed and, when there is a
    source and `with_source`, on the source."""
    bed, source, state0, targets = _keep(bed, source, state0, targets)
    probes, cells = _u32(probes), _u32(cells)
    fd_bed = np.zeros(cells.size)
    fd_src = np.zeros(cells.size) if (source is not None and with_source) else None
    threads = threads or os.cpu_count() or 1
    P = C.POINTER(C.c_uint32)
    lib().oracle_adj_fd(*_grid_args(grid), float(dt), int(ticks), _d(bed), _d(source),
                        _d(state0), probes.ctypes.data_as(P), _d(targets), probes.size,
                        cells.ctypes.data_as(P), cells.size, float(eps_bed), float(rel_source),
                        _d(fd_bed), _d(fd_src), int(threads))
    return fd_bed, fd_src


def adj_loss64(grid: Grid, dt, ticks, bed, source, state0, probes, targets):
    bed, source, state0, targets = _keep(bed, source, state0, targets)
    probes = _u32(probes)
    return float(lib().oracle_adj_loss64(*_grid_args(grid), float(dt), int(ticks), _d(bed),
                                         _d(source), _d(state0),
                                         probes.ctypes.data_as(C.POINTER(C.c_uint32)),
                                         _d(targets), probes.size))


def hash_floats(values) -> int:
    v = np.ascontiguousarray(values, dtype=np.float32)
    return int(lib().oracle_hash_floats(v.ctypes.data_as(_fp), v.size))


# ---- the complete FP64 step (ws_oracle.hpp), and the reference's own build of it ------------

_FULL_FIELDS = dict(depth=0, momentum_x=1, momentum_y=2, ground=3, carried=4, speed=5,
                    bed_stress_x=6, bed_stress_y=7, dissipation=8)
_INPUT_KEYS = ("bed", "manning", "source", "ground_k", "ground_s", "ground_cap")
LEDGER_KEYS = ("source_m3", "open_edge_out_m3", "ground_m3", "roundoff_m3", "scheme_loss_j",
               "friction_work_j", "time_s", "steps")
CARRIED_LEDGER_KEYS = ("source", "from_dissipation", "exchange", "decayed", "open_edge_out")


def _bind_full(L, prefix):
    f = getattr(L, prefix + "create")
    f.restype = C.c_void_p
    f.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_double,
                  C.c_double, C.c_uint32, C.c_uint32, _dp]
    for name, res, args in [("destroy", None, [C.c_void_p]),
                            ("set", None, [C.c_void_p, C.c_int, _dp]),
                            ("get", None, [C.c_void_p, C.c_int, _dp]),
                            ("step", C.c_double, [C.c_void_p, C.c_void_p, C.c_double]),
                            ("advance", C.c_uint64, [C.c_void_p, C.c_void_p, C.c_double]),
                            ("ledger", None, [C.c_void_p, _dp]),
                            ("hash", C.c_uint64, [C.c_void_p])]:
        g = getattr(L, prefix + name)
        g.restype = res
        g.argtypes = args


class FullSolver:
    """water_state::Solver complete (water_state.h:161-266): the oracle's restatement, or with
    reference=True the reference's own build (oracle/_ref, where its sources were present).

    `carried` lists each quantity's (decay_s, per_joule, min_speed_m_per_s). Inputs are a dict:
    bed, manning, source, ground_k, ground_s, ground_cap (arrays or None), carried_source and
    carried_exchange (lists of arrays or None, one a quantity)."""

    def __init__(self, nx, ny, cell_m=1.0, gravity=9.81, cfl=0.45, dry=1e-9, rho=1000.0,
                 open_edges=0, carried=(), reference=False):
        self._L = ref() if reference else lib()
        self._p = "wsref_full_" if reference else "oracle_ws_"
        if not hasattr(self._L, "_full_bound"):
            _bind_full(self._L, self._p)
            self._L._full_bound = True
        self.nx, self.ny, self.k = int(nx), int(ny), len(carried)
        cc = np.zeros(12)
        for i, c in enumerate(carried):
            cc[3 * i:3 * i + 3] = c
        self._cc = cc
        self.h = getattr(self._L, self._p + "create")(self.nx, self.ny, cell_m, gravity, cfl, dry,
                                                      rho, int(open_edges), self.k,
                                                      cc.ctypes.data_as(_dp))

    def __del__(self):
        if getattr(self, "h", None):
            getattr(self._L, self._p + "destroy")(self.h)
            self.h = None

    @property
    def cells(self):
        return self.nx * self.ny

    def _size(self, field):
        return self.cells * (self.k if field == "carried" else 1)

    def set(self, field, values):
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        assert v.size == self._size(field), field
        getattr(self._L, self._p + "set")(self.h, _FULL_FIELDS[field], v.ctypes.data_as(_dp))

    def get(self, field):
        out = np.zeros(self._size(field))
        if out.size:
            getattr(self._L, self._p + "get")(self.h, _FULL_FIELDS[field], out.ctypes.data_as(_dp))
        return out

    def _inputs(self, inputs):
        keep = []
        ptrs = (C.c_void_p * 14)()
        for j, key in enumerate(_INPUT_KEYS):
            a = inputs.get(key)
            if a is not None:
                a = np.ascontiguousarray(a, dtype=np.float64)
                keep.append(a)
                ptrs[j] = a.ctypes.data
        for off, key in ((6, "carried_source"), (10, "carried_exchange")):
            for k, a in enumerate(inputs.get(key) or ()):
                if a is not None:
                    a = np.ascontiguousarray(a, dtype=np.float64)
                    keep.append(a)
                    ptrs[off + k] = a.ctypes.data
        return ptrs, keep

    def step(self, inputs, max_dt):
        ptrs, keep = self._inputs(inputs)
        return getattr(self._L, self._p + "step")(self.h, ptrs, float(max_dt))

    def advance(self, inputs, duration):
        ptrs, keep = self._inputs(inputs)
        return int(getattr(self._L, self._p + "advance")(self.h, ptrs, float(duration)))

    def ledger(self):
        out = np.zeros(28)
        getattr(self._L, self._p + "ledger")(self.h, out.ctypes.data_as(_dp))
        d = dict(zip(LEDGER_KEYS, out[:8]))
        d["steps"] = int(d["steps"])
        d["carried"] = [dict(zip(CARRIED_LEDGER_KEYS, out[8 + 5 * k:13 + 5 * k]))
                        for k in range(self.k)]
        return d

    def state_hash(self):
        return int(getattr(self._L, self._p + "hash")(self.h))


def fd_exp(x):
    """fdlibm's e^x as the oracle restates it (ws_oracle.hpp)."""
    L = lib()
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    L.oracle_fd_exp_n.argtypes = [_dp, _dp, C.c_size_t]
    L.oracle_fd_exp_n(x.ctypes.data_as(_dp), out.ctypes.data_as(_dp), x.size)
    return out


def fd_log(x):
    L = lib()
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    L.oracle_fd_log_n.argtypes = [_dp, _dp, C.c_size_t]
    L.oracle_fd_log_n(x.ctypes.data_as(_dp), out.ctypes.data_as(_dp), x.size)
    return out


def ref_det(name, x):
    """The reference's own det::exp or det::log (core/math/include/core/math/deterministic.h)."""
    R = ref()
    f = getattr(R, f"wsref_det_{name}_n")
    f.argtypes = [_dp, _dp, C.c_size_t]
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    f(x.ctypes.data_as(_dp), out.ctypes.data_as(_dp), x.size)
    return out

"""wlcuda: the reference engine's live-water tick on a GB300 (sm_103a), behind a C ABI.

``libwlcuda.so`` (built by :mod:`game_engine_gb300.buildlib`) holds the CUDA kernels and the C ABI
declared in ``include/wlcuda.h``. :mod:`game_engine_gb300.water_live` mirrors the reference's
``water_live::DeviceStep`` over that ABI; :mod:`game_engine_gb300.batch` the batched tiles and
:mod:`game_engine_gb300.adjoint` the checkpointed reverse tick.

There is no fallback: without the compiled library every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libwlcuda.so")

_lib = None


class LibraryMissing(RuntimeError):
    pass


def lib() -> C.CDLL:
    """The loaded libwlcuda.so; raises LibraryMissing when it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(
                f"{LIB_PATH} is missing: build it with `python -m game_engine_gb300.buildlib` "
                "(nvcc, sm_103a); there is no CPU fallback")
        from . import _abi
        _lib = _abi.bind(C.CDLL(LIB_PATH))
    return _lib


def build(verbose: bool = False) -> str:
    from .buildlib import build as _build
    return _build(verbose=verbose)

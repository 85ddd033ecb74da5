"""Builds libwlcuda.so (the CUDA kernels and the C ABI) in-tree for sm_103a with nvcc.

No contraction and IEEE division and square root in every translation unit of the tick: the step's
bytes must equal the CPU restatement's. The adjoint's unit takes contraction for its reverse march
only (its forward march is spelled in correctly rounded intrinsics throughout). The translation
units compile in parallel; the result lands in ``game_engine_gb300/lib/libwlcuda.so`` (objects in
``game_engine_gb300/_build``).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libwlcuda.so")

SOURCES = ["wl_kernels.cu", "wl_adjoint.cu", "wl_static.cu", "wl_queue.cu", "ws_solver.cu",
           "wl_tiles.cpp", "wl_api.cpp", "wl_batch.cpp", "wl_util.cpp"]
HEADERS = ["wl_device.cuh", "wl_kernels.h", "wl_tiles.h", "wl_adjoint.h", "wl_queue.h",
           "ws_solver.h"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NUMERICS = ["--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
# The adjoint's translation unit: its forward march spells every operation as a correctly rounded
# intrinsic (no contraction can touch it) and its reverse march is a derivative held to a
# tolerance, so contraction is on there.
NUMERICS_BY_SOURCE = {"wl_adjoint.cu": ["--fmad=true", "-prec-div=true", "-prec-sqrt=true",
                                        "-ftz=false"]}
HOST = ["-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math,-Wall"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwlcuda.so")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    cc = nvcc()
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(ROOT, "include", h) for h in ("wlcuda.h", "wlcuda_util.h")]
    procs, objs = [], []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [path] + headers):
            continue
        numerics = NUMERICS_BY_SOURCE.get(src, NUMERICS)
        cmd = [cc, "-std=c++17", "-O3", "-lineinfo", *ARCH, *numerics, *HOST,
               "-I", os.path.join(ROOT, "include"), "-c", path, "-o", obj]
        if src.endswith(".cpp"):
            cmd[1:1] = ["-x", "cu"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(f"--- {s}\n{o}" for s, o in failed))
    if force or procs or _stale(LIB, objs):
        cmd = [cc, "-shared", *ARCH, "-o", LIB + ".tmp", *objs, "-lcudart"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))

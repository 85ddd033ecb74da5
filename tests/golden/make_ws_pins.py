"""Writes tests/golden/ws_full_pins.json: the reference's own water_state::Solver (oracle/_ref,
built from the reference's sources by oracle/build_ref.sh) run on every case of tests/ws_cases.py,
its state hash, its per-run results, and the hashes of its outputs and ledger. The pins let the
oracle's restatement and the device's step be checked where the reference is absent.

    python tests/golden/make_ws_pins.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]

import oracle  # noqa: E402
import ws_cases  # noqa: E402


def digest(a: np.ndarray) -> str:
    """A short digest of an array's bytes (FNV-1a 64 over its 8-byte words' bytes)."""
    h = 0xcbf29ce484222325
    for byte in np.ascontiguousarray(a, dtype=np.float64).tobytes():
        h ^= byte
        h = (h * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return f"{h:016x}"


def main():
    if not oracle.ref_available() and not oracle.build_ref():
        raise SystemExit("the reference's sources are needed")
    pins = {}
    for name, make in sorted(ws_cases.CASES.items()):
        case = make()
        c = case["config"]
        s = oracle.FullSolver(c["nx"], c["ny"], c["cell_m"], open_edges=c["open_edges"],
                              carried=c["carried"], reference=True)
        ws_cases.load(s, case)
        results = ws_cases.run(s, case)
        led = s.ledger()
        pins[name] = dict(results=[float(r) for r in results], state_hash=str(s.state_hash()),
                          outputs={f: digest(s.get(f)) for f in ws_cases.FIELDS},
                          ledger={k: float(v) for k, v in led.items() if k != "carried"},
                          carried_ledger=[{k: float(v) for k, v in d.items()}
                                          for d in led["carried"]])
    with open(os.path.join(HERE, "ws_full_pins.json"), "w") as f:
        json.dump(pins, f, indent=1, sort_keys=True)
        f.write("\n")
    print(f"wrote {len(pins)} cases")


if __name__ == "__main__":
    main()

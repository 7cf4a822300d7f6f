"""Writes tests/golden/roofline_n2p20_k14.json: the reference's own answer for
the roofline-scale instance (random 10-regular graph, n = 2^20, weights in
[1, 1024], k = 14, seed 123456789).

The reference leg of the oracle (oracle/_ref/ref_emv: the unmodified
reader/reader-el.c emv_kernel, R:1966-2139, driven by oracle/ref_harness.c)
solves the whole instance on the host cores -- cost only, int64 f_v of
2^14 x 2^20 cells (128 GiB; about 40 minutes on 16 cores) -- and prints its
cost and the FNV-1a 64 hash of its whole table (int64 values mapped to int32,
INT64_MAX to 2^30, rows in FV_INDEX order X * n + v).  The fixture keeps
those with the instance hash, so the GPU test can check the whole 64 GiB
table without the reference.

Run once on a host with at least 150 GB of free memory:
    python tests/golden/make_roofline_golden.py
"""
from __future__ import annotations

import json
import os
import platform
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

SPEC = {"kind": "regular", "n": 1 << 20, "degree": 10, "wmin": 1, "wmax": 1024, "k": 14, "seed": 123456789}
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "roofline_n2p20_k14.json")
NEED_BYTES = 150 * 10**9


def instance_fnv_fast(orc, inst) -> str:
    """instance_fnv of tests/golden/cases.py (FNV-1a 64 over n, edges and
    terminals as little-endian int64), computed by the oracle's C hash: an
    int64 array viewed as int32 pairs has the same bytes in the same order."""
    words = np.concatenate([np.array([inst.n], np.int64), np.asarray(inst.edges, np.int64).reshape(-1),
                            np.asarray(inst.terminals, np.int64)]).astype("<i8")
    return f"{orc.fnv64(words.view('<i4')):016x}"


def mem_available() -> int:
    with open("/proc/meminfo") as f:
        for line in f:
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    return 0


def main() -> int:
    import oracle
    import steiner_edge_linear_gb300 as E

    if mem_available() < NEED_BYTES:
        print(f"needs {NEED_BYTES / 1e9:.0f} GB of free memory, {mem_available() / 1e9:.0f} GB available")
        return 2
    oracle.build(reference=True)
    if not oracle.reference_available():
        print("reference leg not built")
        return 2
    E.build()
    inst = E.StpInstance.regular(SPEC["n"], SPEC["degree"], SPEC["wmin"], SPEC["wmax"], SPEC["k"], SPEC["seed"])
    threads = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "roofline.stp")
        inst.write(path)
        t0 = time.time()
        r = oracle.ref_emv(path, threads=threads)
        wall = time.time() - t0
    out = {"spec": SPEC, "instance_fnv": instance_fnv_fast(oracle, inst), "n": r["n"], "m": r["m"], "k": r["k"],
           "cost": r["cost"], "table_fnv": f"{r['fnv']:016x}", "inf_cells": r["inf_cells"], "max": r["max"],
           "reference": {"kernel_ms": r["kernel_ms"], "zero_ms": r["zero_ms"], "threads": r["threads"],
                         "wall_s": round(wall, 1), "machine": platform.machine(),
                         "build": "oracle/_ref/ref_emv: -O3 -fopenmp -DBIN_HEAP -DBUILD_PARALLEL"}}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())

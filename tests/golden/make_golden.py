"""Writes tests/golden/golden.json from the reference's own EMV code.

Each case is an instance this repository can regenerate anywhere (the seeded
generator of libemv, or a small hand-written STP file in this folder) plus what
the reference's emv_kernel (reader/reader-el.c:1966-2139, run through
oracle/ref_harness.c) computed on it: the cost, the FNV-1a 64 of the whole
int32 table (INT64_MAX written as 2^30), and for tables up to 2^10 rows the
hash of every row.  An FNV of the instance itself pins the generator, so a
platform whose generator drifted fails loudly instead of comparing the wrong
graph.

Run here, where the reference tree is readable:
    make -C oracle all ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from tests.golden.cases import CASES, instance_for, instance_fnv  # noqa: E402


def main() -> None:
    if not oracle.reference_available():
        raise SystemExit("reference leg not built: make -C oracle ref")
    out = {"generator": "libemv emv_gen_regular / emv_gen_mixed (xoshiro256**, splitmix64 seeding)",
           "reference": "reader/reader-el.c emv_kernel via oracle/ref_harness.c, -DBIN_HEAP -DBUILD_PARALLEL",
           "cases": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for name, spec in CASES.items():
            inst = instance_for(spec)
            path = os.path.join(tmp, name + ".stp")
            inst.write(path)
            rowf = os.path.join(tmp, name + ".rowfnv")
            r = oracle.ref_emv(path, rowfnv_out=rowf)
            entry = {"spec": spec, "n": inst.n, "m": inst.m, "k": inst.k, "instance_fnv": instance_fnv(inst),
                     "cost": r["cost"], "table_fnv": f"{r['fnv']:016x}", "max": r["max"],
                     "inf_cells": r["inf_cells"]}
            if inst.k <= 10:
                rows = np.fromfile(rowf, dtype=np.uint64)
                entry["row_fnv"] = [f"{int(x):016x}" for x in rows]
            out["cases"][name] = entry
            print(f"{name}: n={inst.n} m={inst.m} k={inst.k} cost={r['cost']}", flush=True)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()

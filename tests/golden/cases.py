"""Instances of the golden fixtures and of the parity tests.

A case is a dict: {"kind": "regular", n, degree, wmin, wmax, k, seed},
{"kind": "mixed", base, index} or {"kind": "file", "file": <name in this
folder>, optional "terminals": [...] replacing the file's list}.
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# The measured workload shapes (random regular graphs of the solver's
# benchmark configurations) at sizes the oracle finishes in seconds, plus edge
# cases: k = 1 and 2, ties from tiny weight ranges, zero weights, repeated
# terminals, long paths (many sweeps), stars and dense graphs.
CASES: dict[str, dict] = {
    "plain_n1024_d4_k8": {"kind": "regular", "n": 1024, "degree": 4, "wmin": 1, "wmax": 1000, "k": 8,
                          "seed": 123456789},
    "reg_n64_d3_k4": {"kind": "regular", "n": 64, "degree": 3, "wmin": 1, "wmax": 10, "k": 4, "seed": 1},
    "reg_n100_d4_k6": {"kind": "regular", "n": 100, "degree": 4, "wmin": 1, "wmax": 1000, "k": 6, "seed": 2},
    "reg_n200_d3_k7_ties": {"kind": "regular", "n": 200, "degree": 3, "wmin": 1, "wmax": 3, "k": 7, "seed": 3},
    "reg_n300_d6_k9": {"kind": "regular", "n": 300, "degree": 6, "wmin": 1, "wmax": 1000, "k": 9, "seed": 4},
    "reg_n500_d8_k10": {"kind": "regular", "n": 500, "degree": 8, "wmin": 1, "wmax": 100, "k": 10, "seed": 5},
    "reg_n2000_d20_k6": {"kind": "regular", "n": 2000, "degree": 20, "wmin": 1, "wmax": 100, "k": 6, "seed": 6},
    "reg_n4096_d10_k8": {"kind": "regular", "n": 4096, "degree": 10, "wmin": 1, "wmax": 1024, "k": 8, "seed": 7},
    "reg_n150_d4_k11": {"kind": "regular", "n": 150, "degree": 4, "wmin": 1, "wmax": 50, "k": 11, "seed": 8},
    "reg_n80_d3_k12": {"kind": "regular", "n": 80, "degree": 3, "wmin": 1, "wmax": 20, "k": 12, "seed": 9},
    "reg_zero_w": {"kind": "regular", "n": 256, "degree": 4, "wmin": 0, "wmax": 2, "k": 7, "seed": 10},
    "reg_k1": {"kind": "regular", "n": 50, "degree": 4, "wmin": 1, "wmax": 100, "k": 1, "seed": 11},
    "reg_k2": {"kind": "regular", "n": 400, "degree": 3, "wmin": 1, "wmax": 100, "k": 2, "seed": 12},
    "reg_n33_k3": {"kind": "regular", "n": 34, "degree": 3, "wmin": 1, "wmax": 9, "k": 3, "seed": 13},
    "path_n3000_k5": {"kind": "file", "file": "path3000.stp"},
    "star_n129_k6": {"kind": "file", "file": "star129.stp"},
    "dup_terminals_k5": {"kind": "file", "file": "dup5.stp"},
    "dense_n40_k8": {"kind": "file", "file": "dense40.stp"},
}
for _i in range(24):
    CASES[f"mixed_{_i:02d}"] = {"kind": "mixed", "base": 20240601, "index": _i}


def instance_for(spec: dict):
    """Builds the StpInstance of a case through the product's generator / reader."""
    import steiner_edge_linear_gb300 as E

    kind = spec["kind"]
    if kind == "regular":
        return E.StpInstance.regular(spec["n"], spec["degree"], spec["wmin"], spec["wmax"], spec["k"], spec["seed"])
    if kind == "mixed":
        return E.StpInstance.mixed(spec["base"], spec["index"])
    if kind == "file":
        return E.StpInstance.from_file(os.path.join(HERE, spec["file"]))
    raise ValueError(kind)


def instance_fnv(inst) -> str:
    """FNV-1a 64 of (n, edges, terminals) as int64 little-endian words."""
    h = 1469598103934665603
    data = np.concatenate([np.array([inst.n], np.int64), np.asarray(inst.edges, np.int64).reshape(-1),
                           np.asarray(inst.terminals, np.int64)]).astype("<i8").tobytes()
    for b in data:
        h ^= b
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return f"{h:016x}"

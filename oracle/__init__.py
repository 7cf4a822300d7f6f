"""The oracle: CPU checkers of the GPU EMV solver.

TEST INFRASTRUCTURE ONLY.  tests/, the smoke check of __graft_entry__ and the
CPU-baseline leg of bench.py use this package as the checker; the solver's
product code never imports it.

Two legs:
  * ``emv_table`` -- the C restatement in emv_oracle.c (reader/reader-el.c
    emv_kernel, R:1966-2139, restated), built into _build/liboracle_emv.so;
  * ``ref_emv``   -- the reference's own emv_kernel driven by ref_harness.c,
    built from the unmodified reference source into _ref/ (git-ignored).
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
from typing import Optional

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liboracle_emv.so")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")
REF_EMV = os.path.join(REF_DIR, "ref_emv")
REF_EMV_OPT = os.path.join(REF_DIR, "ref_emv_opt")
REF_READER = os.path.join(REF_DIR, "reader-el")
INF32 = 1 << 30

_lib = None


def build(reference: bool = True) -> None:
    """Compiles the C restatement and, where its source is available, the reference leg."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "all"], check=True)
    if reference:
        r = subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref"], stdout=subprocess.PIPE,
                           stderr=subprocess.STDOUT, text=True)
        if r.returncode not in (0, 2) and "reference source unavailable" not in r.stdout:
            raise RuntimeError("reference build failed:\n" + r.stdout)


def reference_available() -> bool:
    return os.path.exists(REF_EMV) and os.access(REF_EMV, os.X_OK)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(reference=False)
        lib = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        lib.oracle_emv.restype = ctypes.c_int
        lib.oracle_emv.argtypes = [ctypes.c_int32, P, P, P, ctypes.c_int32, P, P, ctypes.POINTER(ctypes.c_int64),
                                   ctypes.c_int32]
        lib.oracle_sssp.restype = ctypes.c_int
        lib.oracle_sssp.argtypes = [ctypes.c_int32, P, P, P, ctypes.c_int32, P]
        lib.oracle_fnv64.restype = ctypes.c_uint64
        lib.oracle_fnv64.argtypes = [P, ctypes.c_int64]
        _lib = lib
    return _lib


def emv_table(n: int, row_ptr: np.ndarray, col: np.ndarray, w: np.ndarray, terminals, threads: int = 0):
    """Full int32 table (2^k, n) and cost by the C restatement."""
    lib = _load()
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
    col = np.ascontiguousarray(col, dtype=np.int32)
    w = np.ascontiguousarray(w, dtype=np.int32)
    t = np.ascontiguousarray(terminals, dtype=np.int32)
    k = int(t.shape[0])
    table = np.empty(((1 << k), n), np.int32)
    cost = ctypes.c_int64()
    st = lib.oracle_emv(n, row_ptr.ctypes.data, col.ctypes.data, w.ctypes.data, k, t.ctypes.data,
                        table.ctypes.data, ctypes.byref(cost), threads)
    if st != 0:
        raise RuntimeError(f"oracle_emv failed with {st}")
    return table, int(cost.value)


def sssp(n: int, row_ptr, col, w, source: int) -> np.ndarray:
    lib = _load()
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
    col = np.ascontiguousarray(col, dtype=np.int32)
    w = np.ascontiguousarray(w, dtype=np.int32)
    d = np.empty(n, np.int64)
    if lib.oracle_sssp(n, row_ptr.ctypes.data, col.ctypes.data, w.ctypes.data, source, d.ctypes.data) != 0:
        raise RuntimeError("oracle_sssp failed")
    return d


def fnv64(a: np.ndarray) -> int:
    a = np.ascontiguousarray(a, dtype=np.int32)
    return int(_load().oracle_fnv64(a.ctypes.data, a.size))


_REF_LINE = re.compile(r"^REF cost=(-?\d+) zero_ms=([\d.]+) kernel_ms=([\d.]+) n=(\d+) m=(\d+) k=(\d+) "
                       r"threads=(\d+) fnv=([0-9a-f]+) inf_cells=(\d+) max=(-?\d+)", re.M)


def ref_emv(stp_path: str, table_out: Optional[str] = None, rowfnv_out: Optional[str] = None,
            kprefix: int = 0, threads: Optional[int] = None, track_optimal: bool = False,
            timeout: Optional[float] = None) -> dict:
    """Runs the reference's emv_kernel on an STP file; returns cost, times and the table hash."""
    exe = REF_EMV_OPT if track_optimal else REF_EMV
    if not os.path.exists(exe):
        raise RuntimeError("reference leg not built (oracle/_ref)")
    cmd = [exe, "-in", stp_path]
    if kprefix:
        cmd += ["-kprefix", str(kprefix)]
    if table_out:
        cmd += ["-table", table_out]
    if rowfnv_out:
        cmd += ["-rowfnv", rowfnv_out]
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=env, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference run failed ({r.returncode}): {r.stderr[-2000:]}")
    mt = _REF_LINE.search(r.stdout)
    if not mt:
        raise RuntimeError("reference output without REF line: " + r.stdout[-2000:])
    g = mt.groups()
    return {"cost": int(g[0]), "zero_ms": float(g[1]), "kernel_ms": float(g[2]), "n": int(g[3]), "m": int(g[4]),
            "k": int(g[5]), "threads": int(g[6]), "fnv": int(g[7], 16), "inf_cells": int(g[8]), "max": int(g[9]),
            "stdout": r.stdout}

"""The oracle: CPU restatements that the GPU EMV solver is compared with.

TEST INFRASTRUCTURE ONLY.  tests/, the smoke check of __graft_entry__ and the
CPU-baseline leg of bench.py use this package as the oracle; the solver's
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
# the reference's shipped test instances, staged by the recipe (Makefile "stage")
TESTSET_DIR = os.path.join(REF_DIR, "testset")
INF32 = 1 << 30
FNV_BASIS = 1469598103934665603

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
        lib.oracle_fnv64_from.restype = ctypes.c_uint64
        lib.oracle_fnv64_from.argtypes = [P, ctypes.c_int64, ctypes.c_uint64]
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


def closure(n: int, row_ptr, col, w, init: np.ndarray) -> np.ndarray:
    """Multi-source closure of each row of init (shape (rows, n), INF32 = no
    value): out[r][v] = min over u of init[r][u] + dist(u, v), as int64 with
    INF32 where nothing reaches v.  Each row is one Dijkstra (oracle_sssp)
    from a virtual source whose arcs to u weigh init[r][u] -- the reference's
    virtual-source relaxation (reader-el.c:2090-2116)."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int64)
    w = np.ascontiguousarray(w, dtype=np.int64)
    arcs = int(row_ptr[n])
    out = np.empty(init.shape, np.int64)
    for r in range(init.shape[0]):
        src = np.nonzero(init[r] < INF32)[0]
        rp = np.concatenate([row_ptr, [arcs + src.size]]).astype(np.int32)
        cc = np.concatenate([col[:arcs], src]).astype(np.int32)
        ww = np.concatenate([w[:arcs], init[r][src].astype(np.int64)]).astype(np.int32)
        d = sssp(n + 1, rp, cc, ww, n)[:n]
        out[r] = np.where(d == np.iinfo(np.int64).max, INF32, d)
    return out


def fnv64(a: np.ndarray, h: int = FNV_BASIS) -> int:
    """FNV-1a 64 of the int32 words' bytes; pass the previous result as h to
    hash a table piece by piece (the reference harness hashes it whole)."""
    a = np.ascontiguousarray(a, dtype=np.int32)
    return int(_load().oracle_fnv64_from(a.ctypes.data, a.size, h))


def read_stp_csr(path: str):
    """(n, row_ptr, col, w, terminals) of an STP file, int32, 0-based, with
    the arcs in the order root_build fills them (reader-el.c:794-826: edge
    order, both arcs of every edge).  Reads only what the solver's own writer
    emits ("e u v w" and "t v" lines), for CPU baselines that must not load
    the solver's library."""
    n = 0
    edges, terms = [], []
    with open(path) as f:
        for line in f:
            tok = line.split()
            if not tok:
                continue
            if tok[0] == "nodes":
                n = int(tok[1])
            elif tok[0] == "e" and len(tok) >= 4:
                edges.append((int(tok[1]) - 1, int(tok[2]) - 1, int(tok[3])))
            elif tok[0] == "t" and len(tok) >= 2:
                terms.append(int(tok[1]) - 1)
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 3)
    src = np.stack([e[:, 0], e[:, 1]], axis=1).reshape(-1)
    dst = np.stack([e[:, 1], e[:, 0]], axis=1).reshape(-1)
    wt = np.repeat(e[:, 2], 2)
    order = np.argsort(src, kind="stable")
    row_ptr = np.zeros(n + 1, np.int32)
    np.cumsum(np.bincount(src, minlength=n), out=row_ptr[1:])
    return (n, row_ptr, dst[order].astype(np.int32), wt[order].astype(np.int32),
            np.asarray(terms, dtype=np.int32))


def testset_files() -> list:
    """The reference's 204 SteinLib and 3 path instances (staged copies), or []."""
    import glob

    files = sorted(glob.glob(os.path.join(TESTSET_DIR, "small-instances", "*", "*.stp")))
    files += sorted(glob.glob(os.path.join(TESTSET_DIR, "path", "*.stp")))
    return files


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

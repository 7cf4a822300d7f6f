"""GB300-native Erickson-Monma-Veinott Steiner solver.

Python face of the C ABI in ``include/emv.h`` (loaded with ctypes from the
in-tree ``lib/libemv.so``).  The names mirror the reference solver's own
functions in reader/reader-el.c:

  ``graph_load(path)``              -> graph_load          (R:473-618)
  ``root_build(g)``                 -> root_build          (R:706-899)
  ``erickson_monma_veinott(r, l)``  -> erickson_monma_veinott (R:2141-2343)
  ``Solver.kernel_dev(...)``        -> emv_kernel          (R:1966-2139)
  ``Solver.sssp(...)``              -> dijkstra            (R:1762-1880)

There is no CPU fallback: every solve runs the sm_103a kernels, and loading
fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import build as _build

INF32 = 1 << 30
LIB_PATH = _build.LIB_PATH
CLI_PATH = _build.CLI_PATH

BATCH_CLASSES = 12
TREE = 0x1
TABLE = 0x2
NOCHECK = 0x4

STATUS = {
    0: "EMV_OK", 1: "EMV_ERR_BAD_INPUT", 2: "EMV_ERR_PARSE", 3: "EMV_ERR_OOM", 4: "EMV_ERR_OVER_BUDGET",
    5: "EMV_ERR_TIMEOUT", 6: "EMV_ERR_CUDA", 7: "EMV_ERR_DISCONNECTED", 8: "EMV_ERR_OVERFLOW",
    9: "EMV_ERR_NOT_READY", 10: "EMV_ERR_CANCELLED", 11: "EMV_ERR_INTERNAL",
}
ERR_NOT_READY = 9


class EmvError(RuntimeError):
    """A non-zero emv status, with the library's message."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


# ----------------------------------------------------------------- C structs

class _Stp(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("m", ctypes.c_int64), ("k", ctypes.c_int64), ("cost", ctypes.c_int64),
                ("edges", ctypes.POINTER(ctypes.c_int64)), ("terminals", ctypes.POINTER(ctypes.c_int64))]


class _Graph(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("arcs", ctypes.c_int64), ("row_ptr", ctypes.c_void_p),
                ("col", ctypes.c_void_p), ("w", ctypes.c_void_p)]


class _Timing(ctypes.Structure):
    _fields_ = [("zero_ms", ctypes.c_float), ("level1_ms", ctypes.c_float), ("merge_ms", ctypes.c_float),
                ("relax_ms", ctypes.c_float), ("traceback_ms", ctypes.c_float), ("kernel_ms", ctypes.c_float),
                ("relax_sweeps", ctypes.c_int64), ("launches", ctypes.c_int64), ("relax16_levels", ctypes.c_int64),
                ("merge16_levels", ctypes.c_int64), ("relax_launches", ctypes.c_int64)]


class _Result(ctypes.Structure):
    _fields_ = [("cost", ctypes.c_int64), ("tree", ctypes.c_void_p), ("tree_cap", ctypes.c_int64),
                ("tree_count", ctypes.c_int64), ("tree_weight", ctypes.c_int64), ("table", ctypes.c_void_p),
                ("timing", _Timing)]


class _Instance(ctypes.Structure):
    _fields_ = [("g", _Graph), ("terminals", ctypes.c_void_p), ("k", ctypes.c_int32)]


_INSTANCE_DTYPE = np.dtype({"names": ["n", "arcs", "row_ptr", "col", "w", "terminals", "k"],
                            "formats": ["<i4", "<i8", "<u8", "<u8", "<u8", "<u8", "<i4"],
                            "offsets": [_Instance.g.offset + _Graph.n.offset, _Instance.g.offset + _Graph.arcs.offset,
                                        _Instance.g.offset + _Graph.row_ptr.offset,
                                        _Instance.g.offset + _Graph.col.offset, _Instance.g.offset + _Graph.w.offset,
                                        _Instance.terminals.offset, _Instance.k.offset],
                            "itemsize": ctypes.sizeof(_Instance)})


class _BatchStats(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_float), ("upload_ms", ctypes.c_float), ("work_items", ctypes.c_int64),
                ("table_bytes", ctypes.c_int64), ("merge_tile", ctypes.c_int32), ("relax_rows", ctypes.c_int32)]


class _ServerOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64), ("max_slots", ctypes.c_int32),
                ("large_n", ctypes.c_int32), ("wave_sms", ctypes.c_int32)]


class _ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("rejected", ctypes.c_int64),
                ("waves", ctypes.c_int64), ("peak_resident", ctypes.c_int64), ("peak_bytes", ctypes.c_int64)]


_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64

# name -> (restype, argtypes); the list of exported entry points of include/emv.h
SIGNATURES = {
    "emv_status_str": (ctypes.c_char_p, [ctypes.c_int]),
    "emv_last_error": (ctypes.c_char_p, []),
    "emv_version": (ctypes.c_char_p, []),
    "emv_stp_parse": (ctypes.c_int, [ctypes.c_char_p, _I64, ctypes.POINTER(ctypes.POINTER(_Stp))]),
    "emv_stp_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(_Stp))]),
    "emv_stp_free": (None, [ctypes.POINTER(_Stp)]),
    "emv_stp_write": (ctypes.c_int, [ctypes.POINTER(_Stp), ctypes.c_char_p]),
    "emv_csr_build": (ctypes.c_int, [_I64, _I64, _P, _P, _P, _P]),
    "emv_graph_check": (ctypes.c_int, [ctypes.POINTER(_Graph), ctypes.POINTER(_I64)]),
    "emv_gen_regular": (ctypes.c_int, [_I64, _I32, _I32, _I32, _I32, _U64, ctypes.POINTER(ctypes.POINTER(_Stp))]),
    "emv_gen_mixed": (ctypes.c_int, [_U64, _I64, _I32, _I32, _I32, _I32, _I32,
                                     ctypes.POINTER(ctypes.POINTER(_Stp))]),
    "emv_gen_powlaw": (ctypes.c_int, [_I64, _I32, ctypes.c_double, _I32, _I32, _I32, _I32, _U64,
                                      ctypes.POINTER(ctypes.POINTER(_Stp))]),
    "emv_gen_clique": (ctypes.c_int, [_I64, _I32, _I32, _I32, _U64, ctypes.POINTER(ctypes.POINTER(_Stp))]),
    "emv_create": (ctypes.c_int, [ctypes.POINTER(_P), _I32]),
    "emv_destroy": (ctypes.c_int, [_P]),
    "emv_set_sweep_limit": (ctypes.c_int, [_P, _I64]),
    "emv_set_value_bits": (ctypes.c_int, [_P, ctypes.c_int32]),
    "emv_kernel_dev": (ctypes.c_int, [_P, _I32, _I64, _P, _P, _P, _I32, _P, _P, _I64, ctypes.POINTER(_I64), _P]),
    "emv_solve": (ctypes.c_int, [_P, ctypes.POINTER(_Graph), _P, _I32, _I32, ctypes.POINTER(_Result), _P]),
    "emv_solve_dev": (ctypes.c_int, [_P, ctypes.POINTER(_Graph), _P, _I32, _I32, ctypes.POINTER(_Result), _P]),
    "emv_sssp": (ctypes.c_int, [_P, ctypes.POINTER(_Graph), _I32, _P, ctypes.POINTER(ctypes.c_float), _P]),
    "emv_closure_noalloc": (ctypes.c_int, [_I32, _I64, _P, _P, _P, _P, _I32, _I64, _P, _P]),
    "emv_batch_solve": (ctypes.c_int, [_P, ctypes.POINTER(_Instance), _I32, _P, ctypes.POINTER(_BatchStats), _P]),
    "emv_batch_solve_tables": (ctypes.c_int, [_P, ctypes.POINTER(_Instance), _I32, _P, _P,
                                              ctypes.POINTER(_BatchStats), _P]),
    "emv_batch_autotune": (ctypes.c_int, [_P, ctypes.POINTER(_Instance), _I32, _P, _P]),
    "emv_batch_set_tuning": (ctypes.c_int, [_P, _P, _I32]),
    "emv_batch_autotune2": (ctypes.c_int, [_P, ctypes.POINTER(_Instance), _I32, _P, _P, _P]),
    "emv_batch_set_tuning2": (ctypes.c_int, [_P, _P, _P, _I32]),
    "emv_server_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.POINTER(_ServerOpts)]),
    "emv_server_submit": (ctypes.c_int, [_P, ctypes.POINTER(_Graph), _P, _I32, ctypes.POINTER(_I64)]),
    "emv_server_poll": (ctypes.c_int, [_P, _I64, ctypes.POINTER(_I64), ctypes.POINTER(ctypes.c_double)]),
    "emv_server_wait": (ctypes.c_int, [_P, _I64, ctypes.POINTER(_I64), ctypes.POINTER(ctypes.c_double),
                                       ctypes.c_double]),
    "emv_server_cancel": (ctypes.c_int, [_P, _I64]),
    "emv_server_stats_get": (ctypes.c_int, [_P, ctypes.POINTER(_ServerStats)]),
    "emv_server_destroy": (ctypes.c_int, [_P]),
    "emv_bin_write": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(_Stp)), _I32, _I32]),
    "emv_bin_open": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_P)]),
    "emv_bin_count": (_I32, [_P]),
    "emv_bin_instance": (ctypes.c_int, [_P, _I32, ctypes.POINTER(_Instance), ctypes.POINTER(_I64)]),
    "emv_bin_stp": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.POINTER(_Stp))]),
    "emv_bin_close": (None, [_P]),
}

_lib: Optional[ctypes.CDLL] = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads libemv.so once and declares every entry point; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA library first "
                           "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(status: int) -> None:
    if status != 0:
        msg = load_library().emv_last_error().decode(errors="replace")
        raise EmvError(status, msg)


def _ptr(a: Optional[np.ndarray]) -> Optional[int]:
    return None if a is None else a.ctypes.data


# ------------------------------------------------------------------ instances

@dataclass
class StpInstance:
    """A parsed or generated instance (the reference's graph_t, R:358-373)."""

    n: int
    edges: np.ndarray      # (m, 3) int64: u, v, w, 0-based
    terminals: np.ndarray  # (k,) int64, 0-based
    cost: int = -1

    @property
    def m(self) -> int:
        return int(self.edges.shape[0])

    @property
    def k(self) -> int:
        return int(self.terminals.shape[0])

    @staticmethod
    def _take(p) -> "StpInstance":
        lib = load_library()
        s = p.contents
        edges = np.ctypeslib.as_array(s.edges, shape=(int(s.m) * 3,)).reshape(-1, 3).copy() if s.m else \
            np.zeros((0, 3), np.int64)
        terms = np.ctypeslib.as_array(s.terminals, shape=(int(s.k),)).copy() if s.k else np.zeros(0, np.int64)
        out = StpInstance(int(s.n), edges, terms, int(s.cost))
        lib.emv_stp_free(p)
        return out

    @staticmethod
    def from_file(path: str) -> "StpInstance":
        p = ctypes.POINTER(_Stp)()
        _check(load_library().emv_stp_load(path.encode(), ctypes.byref(p)))
        return StpInstance._take(p)

    @staticmethod
    def from_text(text: str | bytes) -> "StpInstance":
        b = text.encode() if isinstance(text, str) else text
        p = ctypes.POINTER(_Stp)()
        _check(load_library().emv_stp_parse(b, len(b), ctypes.byref(p)))
        return StpInstance._take(p)

    @staticmethod
    def regular(n: int, degree: int, wmin: int, wmax: int, k: int, seed: int) -> "StpInstance":
        """Random d-regular instance (configuration model, connected; emv_gen_regular)."""
        p = ctypes.POINTER(_Stp)()
        _check(load_library().emv_gen_regular(n, degree, wmin, wmax, k, seed, ctypes.byref(p)))
        return StpInstance._take(p)

    @staticmethod
    def mixed(base_seed: int, index: int, nmin: int = 64, nmax: int = 4096, kmin: int = 4, kmax: int = 10,
              group_pct: int = 10) -> "StpInstance":
        """Instance ``index`` of the mixed batched distribution (emv_gen_mixed)."""
        p = ctypes.POINTER(_Stp)()
        _check(load_library().emv_gen_mixed(base_seed, index, nmin, nmax, kmin, kmax, group_pct, ctypes.byref(p)))
        return StpInstance._take(p)

    @staticmethod
    def powlaw(n: int, degree: int, alpha: float, classes: int, wmin: int, wmax: int, k: int,
               seed: int) -> "StpInstance":
        """Power-law random instance (emv_gen_powlaw)."""
        p = ctypes.POINTER(_Stp)()
        _check(load_library().emv_gen_powlaw(n, degree, alpha, classes, wmin, wmax, k, seed, ctypes.byref(p)))
        return StpInstance._take(p)

    @staticmethod
    def clique(n: int, wmin: int, wmax: int, k: int, seed: int) -> "StpInstance":
        """Complete-graph instance (emv_gen_clique)."""
        p = ctypes.POINTER(_Stp)()
        _check(load_library().emv_gen_clique(n, wmin, wmax, k, seed, ctypes.byref(p)))
        return StpInstance._take(p)

    def write(self, path: str) -> None:
        e = np.ascontiguousarray(self.edges, dtype=np.int64).reshape(-1)
        t = np.ascontiguousarray(self.terminals, dtype=np.int64)
        s = _Stp(self.n, self.m, self.k, self.cost, e.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                 t.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        _check(load_library().emv_stp_write(ctypes.byref(s), path.encode()))


@dataclass
class Csr:
    """Host int32 CSR with both arcs of every edge (root_build, R:706-899)."""

    n: int
    row_ptr: np.ndarray
    col: np.ndarray
    w: np.ndarray
    terminals: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    cost: int = -1

    @property
    def arcs(self) -> int:
        return int(self.col.shape[0])

    @property
    def k(self) -> int:
        return int(self.terminals.shape[0])

    @staticmethod
    def from_stp(g: StpInstance) -> "Csr":
        n, m = g.n, g.m
        row = np.zeros(n + 1, np.int32)
        col = np.zeros(max(2 * m, 1), np.int32)
        w = np.zeros(max(2 * m, 1), np.int32)
        e = np.ascontiguousarray(g.edges, dtype=np.int64).reshape(-1)
        _check(load_library().emv_csr_build(n, m, _ptr(e), _ptr(row), _ptr(col), _ptr(w)))
        return Csr(n, row, col[:2 * m], w[:2 * m], np.ascontiguousarray(g.terminals, dtype=np.int32), g.cost)

    def _ptrs(self) -> tuple:
        """(n, arcs, row_ptr, col, w, terminals, k) with data addresses, cached
        while the same array objects stay attached (in-place edits keep them)."""
        arrays = (self.row_ptr, self.col, self.w, self.terminals)
        c = self.__dict__.get("_ptr_cache")
        # the cache holds the array objects themselves, so an identity match is
        # the same live buffers
        if c is None or self.n != c[1][0] or any(x is not y for x, y in zip(arrays, c[0])):
            c = (arrays, (self.n, int(self.col.shape[0]), self.row_ptr.ctypes.data, self.col.ctypes.data,
                          self.w.ctypes.data, self.terminals.ctypes.data, int(self.terminals.shape[0])))
            self.__dict__["_ptr_cache"] = c
        return c[1]

    def c_graph(self) -> _Graph:
        return _Graph(self.n, self.arcs, _ptr(self.row_ptr), _ptr(self.col), _ptr(self.w))

    def check(self) -> int:
        """Connectivity and int32-range check (emv_graph_check); returns the value bound."""
        b = ctypes.c_int64()
        g = self.c_graph()
        _check(load_library().emv_graph_check(ctypes.byref(g), ctypes.byref(b)))
        return int(b.value)


class BinContainer:
    """EMVBIN01 container of instances in solver form (emv_bin_*): int32 CSR,
    terminals, cost and optionally the STP edge list.  The reference's
    experiment driver passes "-bin" (experiments/report.py:265-266) but has no
    binary reader; this format is the solver's own."""

    def __init__(self, path: str):
        self._lib = load_library()
        self._b = ctypes.c_void_p()
        _check(self._lib.emv_bin_open(path.encode(), ctypes.byref(self._b)))

    @staticmethod
    def write(path: str, instances: Sequence["StpInstance"], with_edges: bool = True) -> None:
        keep = []
        arr = (ctypes.POINTER(_Stp) * len(instances))()
        for i, g in enumerate(instances):
            e = np.ascontiguousarray(g.edges, dtype=np.int64).reshape(-1)
            t = np.ascontiguousarray(g.terminals, dtype=np.int64)
            st = _Stp(g.n, g.m, g.k, g.cost, e.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                      t.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
            keep.append((e, t, st))
            arr[i] = ctypes.pointer(st)
        _check(load_library().emv_bin_write(path.encode(), arr, len(instances), int(bool(with_edges))))

    def __len__(self) -> int:
        return int(self._lib.emv_bin_count(self._b))

    def csr(self, index: int) -> "Csr":
        """Instance `index` as a Csr (arrays copied out of the container)."""
        inst = _Instance()
        cost = ctypes.c_int64()
        _check(self._lib.emv_bin_instance(self._b, index, ctypes.byref(inst), ctypes.byref(cost)))
        n, arcs, k = int(inst.g.n), int(inst.g.arcs), int(inst.k)

        def view(ptr, count):
            return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_int32)), shape=(count,)).copy()

        empty = np.zeros(0, np.int32)
        return Csr(n, view(inst.g.row_ptr, n + 1), view(inst.g.col, arcs) if arcs else empty,
                   view(inst.g.w, arcs) if arcs else empty, view(inst.terminals, k), int(cost.value))

    def stp(self, index: int) -> "StpInstance":
        """Instance `index` in STP form (needs the edge list in the container)."""
        p = ctypes.POINTER(_Stp)()
        _check(self._lib.emv_bin_stp(self._b, index, ctypes.byref(p)))
        return StpInstance._take(p)

    def close(self) -> None:
        if self._b:
            self._lib.emv_bin_close(self._b)
            self._b = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Result:
    cost: int
    tree: Optional[np.ndarray]      # (count, 3) int32: u, v, w
    tree_weight: int
    table: Optional[np.ndarray]     # (2^k, n) int32
    timing: dict


def _timing(t: _Timing) -> dict:
    return {f: getattr(t, f) for f, _ in _Timing._fields_}


class Solver:
    """A solver context on one CUDA device (emv_create / emv_destroy)."""

    def __init__(self, device: int = 0):
        self._lib = load_library()
        self._ctx = ctypes.c_void_p()
        _check(self._lib.emv_create(ctypes.byref(self._ctx), device))

    def close(self) -> None:
        if self._ctx:
            self._lib.emv_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self) -> "Solver":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def solve(self, g: Csr, terminals: Optional[Sequence[int]] = None, tree: bool = False, table: bool = False,
              check: bool = True, stream: Optional[int] = None) -> Result:
        """erickson_monma_veinott on a host CSR (emv_solve)."""
        terms = np.ascontiguousarray(g.terminals if terminals is None else terminals, dtype=np.int32)
        k = int(terms.shape[0])
        res = _Result()
        tree_buf = np.zeros((g.n + 1, 3), np.int32) if tree else None
        tab = np.zeros(((1 << k), g.n), np.int32) if table and k <= 24 else None
        if tree_buf is not None:
            res.tree = tree_buf.ctypes.data
            res.tree_cap = g.n + 1
        if tab is not None:
            res.table = tab.ctypes.data
        flags = (TREE if tree else 0) | (TABLE if table else 0) | (0 if check else NOCHECK)
        cg = g.c_graph()
        _check(self._lib.emv_solve(self._ctx, ctypes.byref(cg), terms.ctypes.data, k, flags, ctypes.byref(res),
                                   stream))
        tr = tree_buf[:res.tree_count].copy() if tree_buf is not None else None
        return Result(int(res.cost), tr, int(res.tree_weight), tab, _timing(res.timing))

    def solve_dev(self, n: int, arcs: int, row_ptr: int, col: int, w: int, terminals: Sequence[int],
                  tree: bool = False, stream: Optional[int] = None) -> Result:
        """emv_solve_dev on device pointers (e.g. torch tensors' data_ptr())."""
        terms = np.ascontiguousarray(terminals, dtype=np.int32)
        res = _Result()
        tree_buf = np.zeros((n + 1, 3), np.int32) if tree else None
        if tree_buf is not None:
            res.tree = tree_buf.ctypes.data
            res.tree_cap = n + 1
        cg = _Graph(n, arcs, row_ptr, col, w)
        _check(self._lib.emv_solve_dev(self._ctx, ctypes.byref(cg), terms.ctypes.data, int(terms.shape[0]),
                                       TREE if tree else 0, ctypes.byref(res), stream))
        tr = tree_buf[:res.tree_count].copy() if tree_buf is not None else None
        return Result(int(res.cost), tr, int(res.tree_weight), None, _timing(res.timing))

    def set_sweep_limit(self, limit: int) -> None:
        """Caps the relaxation sweeps per chunk (0 = the Bellman-Ford bound); a
        solve that hits the cap raises EmvError with EMV_ERR_TIMEOUT."""
        _check(self._lib.emv_set_sweep_limit(self._ctx, int(limit)))

    def set_value_bits(self, bits: int) -> None:
        """Width of the values in the merge's staged rows and the relaxation's
        records: 0 = 16 bits where the level maxima allow, 32 = always 32."""
        _check(self._lib.emv_set_value_bits(self._ctx, int(bits)))

    def kernel_dev(self, n: int, arcs: int, row_ptr: int, col: int, w: int, terminals: Sequence[int],
                   table: int, ld: int, stream: Optional[int] = None) -> int:
        """emv_kernel on device data and a caller-owned device table (emv_kernel_dev)."""
        terms = np.ascontiguousarray(terminals, dtype=np.int32)
        cost = ctypes.c_int64()
        _check(self._lib.emv_kernel_dev(self._ctx, n, arcs, row_ptr, col, w, int(terms.shape[0]),
                                        terms.ctypes.data, table, ld, ctypes.byref(cost), stream))
        return int(cost.value)

    def sssp(self, g: Csr, source: int, stream: Optional[int] = None) -> tuple[np.ndarray, float]:
        """Single-source distances (the -dijkstra command); INT64_MAX = unreachable."""
        dist = np.zeros(g.n, np.int64)
        ms = ctypes.c_float()
        cg = g.c_graph()
        _check(self._lib.emv_sssp(self._ctx, ctypes.byref(cg), source, dist.ctypes.data, ctypes.byref(ms), stream))
        return dist, float(ms.value)

    @staticmethod
    def _instances(graphs: Sequence[Csr]):
        """emv_instance array of the graphs, filled column-wise through a numpy
        view of the same layout (much cheaper than per-field ctypes stores)."""
        arr = np.zeros(len(graphs), _INSTANCE_DTYPE)
        if graphs:
            cols = list(zip(*(g._ptrs() for g in graphs)))
            for name, col in zip(("n", "arcs", "row_ptr", "col", "w", "terminals", "k"), cols):
                arr[name] = col
        return arr.ctypes.data_as(ctypes.POINTER(_Instance)), arr

    def batch_autotune(self, graphs: Sequence[Csr], stream: Optional[int] = None) -> np.ndarray:
        """Tunes the batched launch per instance class (emv_batch_autotune); returns the rcap table."""
        insts, _keep = self._instances(graphs)
        out = np.zeros(BATCH_CLASSES, np.int32)
        _check(self._lib.emv_batch_autotune(self._ctx, insts, len(graphs), out.ctypes.data, stream))
        return out

    def batch_set_tuning(self, rcap) -> None:
        r = np.ascontiguousarray(rcap, dtype=np.int32)
        _check(self._lib.emv_batch_set_tuning(self._ctx, r.ctypes.data, int(r.shape[0])))

    def batch_autotune_tiles(self, graphs: Sequence[Csr], stream: Optional[int] = None):
        """Tunes the relaxation rows per chunk and the merge vertex-block width
        per instance class (emv_batch_autotune2); returns (rcap, mw) tables."""
        insts, _keep = self._instances(graphs)
        rcap = np.zeros(BATCH_CLASSES, np.int32)
        mw = np.zeros(BATCH_CLASSES, np.int32)
        _check(self._lib.emv_batch_autotune2(self._ctx, insts, len(graphs), rcap.ctypes.data, mw.ctypes.data, stream))
        return rcap, mw

    def batch_set_tiles(self, rcap, mw) -> None:
        """Installs both tuning tables (emv_batch_set_tuning2)."""
        r = np.ascontiguousarray(rcap, dtype=np.int32)
        w = np.ascontiguousarray(mw, dtype=np.int32)
        _check(self._lib.emv_batch_set_tuning2(self._ctx, r.ctypes.data, w.ctypes.data, int(r.shape[0])))

    @staticmethod
    def closure_noalloc(n: int, arcs: int, row_ptr: int, col: int, w: int, init: int, rows: int, ld: int,
                        out: int, stream: Optional[int] = None) -> None:
        """Shortest-path closure of up to 32 device rows with no device allocation (emv_closure_noalloc)."""
        _check(load_library().emv_closure_noalloc(n, arcs, row_ptr, col, w, init, rows, ld, out, stream))

    def batch_solve(self, graphs: Sequence[Csr], stream: Optional[int] = None, tables: bool = False):
        """Many independent instances in one persistent launch (emv_batch_solve);
        with tables=True also every instance's (2^k, n) table
        (emv_batch_solve_tables) as a third return value."""
        count = len(graphs)
        insts, _keep = self._instances(graphs)
        costs = np.zeros(count, np.int64)
        st = _BatchStats()
        if not tables:
            _check(self._lib.emv_batch_solve(self._ctx, insts, count, costs.ctypes.data, ctypes.byref(st), stream))
            return costs, {f: getattr(st, f) for f, _ in _BatchStats._fields_}
        tabs = [np.empty(((1 << g.k), g.n), np.int32) for g in graphs]
        ptrs = (ctypes.c_void_p * max(count, 1))(*[t.ctypes.data for t in tabs])
        _check(self._lib.emv_batch_solve_tables(self._ctx, insts, count, costs.ctypes.data, ptrs,
                                                ctypes.byref(st), stream))
        return costs, {f: getattr(st, f) for f, _ in _BatchStats._fields_}, tabs


class Server:
    """Continuous-batching request loop on one GPU (emv_server_*)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 150 * 10**9, max_slots: int = 4096,
                 large_n: int = 65536, wave_sms: int = 0):
        """wave_sms: SMs kept for the small requests while a large one runs
        (0: a sixth of the SMs; negative: no split)."""
        self._lib = load_library()
        self._srv = ctypes.c_void_p()
        opts = _ServerOpts(device, hbm_budget_bytes, max_slots, large_n, wave_sms)
        _check(self._lib.emv_server_create(ctypes.byref(self._srv), ctypes.byref(opts)))
        self._keep: dict[int, Csr] = {}

    def submit(self, g: Csr) -> int:
        rid = ctypes.c_int64()
        cg = g.c_graph()
        _check(self._lib.emv_server_submit(self._srv, ctypes.byref(cg), g.terminals.ctypes.data, g.k,
                                           ctypes.byref(rid)))
        return int(rid.value)

    def poll(self, rid: int) -> Optional[tuple[int, float]]:
        cost = ctypes.c_int64()
        lat = ctypes.c_double()
        st = self._lib.emv_server_poll(self._srv, rid, ctypes.byref(cost), ctypes.byref(lat))
        if st == ERR_NOT_READY:
            return None
        _check(st)
        return int(cost.value), float(lat.value)

    def wait(self, rid: int, timeout_s: float = 600.0) -> tuple[int, float]:
        cost = ctypes.c_int64()
        lat = ctypes.c_double()
        _check(self._lib.emv_server_wait(self._srv, rid, ctypes.byref(cost), ctypes.byref(lat), timeout_s))
        return int(cost.value), float(lat.value)

    def cancel(self, rid: int) -> None:
        _check(self._lib.emv_server_cancel(self._srv, rid))

    def stats(self) -> dict:
        s = _ServerStats()
        _check(self._lib.emv_server_stats_get(self._srv, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in _ServerStats._fields_}

    def close(self) -> None:
        if self._srv:
            self._lib.emv_server_destroy(self._srv)
            self._srv = ctypes.c_void_p()

    def __enter__(self) -> "Server":
        return self

    def __exit__(self, *exc) -> None:
        self.close()


# ------------------------------------------------- reference-named entry points

def graph_load(path: Optional[str]) -> StpInstance:
    """graph_load (R:473-618); None reads stdin."""
    if path is None:
        import sys
        return StpInstance.from_text(sys.stdin.buffer.read())
    return StpInstance.from_file(path)


def root_build(g: StpInstance) -> Csr:
    """root_build (R:706-899): CSR plus the terminal index kk."""
    return Csr.from_stp(g)


def erickson_monma_veinott(root: Csr, list_soln: bool = False, solver: Optional[Solver] = None) -> Result:
    """erickson_monma_veinott (R:2141-2343) on the GPU."""
    own = solver is None
    s = Solver() if own else solver
    try:
        return s.solve(root, tree=list_soln)
    finally:
        if own:
            s.close()


def build() -> str:
    """Compiles the native library and command in-tree (sm_103a)."""
    return _build.build()

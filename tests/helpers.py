"""Shared checks of the test suite."""
from __future__ import annotations

import numpy as np


def table_row_fnv(table: np.ndarray) -> list[str]:
    """FNV-1a 64 of each int32 row (little-endian bytes), as hex strings."""
    out = []
    for row in np.ascontiguousarray(table, dtype="<i4"):
        h = 1469598103934665603
        for b in row.tobytes():
            h ^= b
            h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
        out.append(f"{h:016x}")
    return out


def check_tree(n: int, edges_uvw: np.ndarray, tree: np.ndarray, terminals, cost: int) -> None:
    """A valid Steiner tree: real input edges (with their weights), acyclic,
    connected, spanning every terminal, total weight equal to the cost.  This
    is stricter than the reference's own check (experiments/verify.py:104-118,
    connectivity and terminal coverage only)."""
    import networkx as nx

    k = len(terminals)
    if k <= 1:
        assert len(tree) == 0
        return
    best = {}
    for u, v, w in np.asarray(edges_uvw, dtype=np.int64):
        key = (min(u, v), max(u, v))
        best.setdefault(key, set()).add(int(w))
    G = nx.Graph()
    total = 0
    for u, v, w in np.asarray(tree, dtype=np.int64):
        key = (min(u, v), max(u, v))
        assert key in best, f"tree edge {u}-{v} is not an input edge"
        assert int(w) in best[key], f"tree edge {u}-{v} weight {w} not an input weight"
        assert not G.has_edge(u, v), "duplicate tree edge"
        G.add_edge(int(u), int(v))
        total += int(w)
    terms = set(int(t) for t in terminals)
    if len(terms) == 1:
        assert total == cost
        return
    assert all(t in G for t in terms), "tree misses a terminal"
    assert nx.is_tree(G), "edges do not form a tree"
    assert total == cost, f"tree weight {total} != cost {cost}"

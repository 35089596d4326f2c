"""Seeded neighbour lists for the general-graph tests (CSR with sorted rows)."""
import numpy as np


def from_edges(n, edges, values=None):
    """Symmetric CSR (rowptr, col, val-or-None) from undirected edges (u != v)."""
    rows = [[] for _ in range(n)]
    for k, (u, v) in enumerate(edges):
        w = None if values is None else float(values[k])
        rows[u].append((v, w))
        rows[v].append((u, w))
    rowptr = np.zeros(n + 1, np.int64)
    col, val = [], []
    for v in range(n):
        r = sorted(rows[v])
        col += [c for c, _ in r]
        val += [w for _, w in r]
        rowptr[v + 1] = len(col)
    return rowptr, np.asarray(col, np.int32), (None if values is None else np.asarray(val, np.float64))


def grid_edges(dims, periodic):
    """Edges of a hyper-cubic grid, first coordinate fastest (sorted, deduplicated)."""
    n = int(np.prod(dims))
    es = set()
    stride = 1
    for L in dims:
        for v in range(n):
            x = (v // stride) % L
            if x + 1 < L:
                u = v + stride
            elif periodic and L > 1:
                u = v - (L - 1) * stride
            else:
                continue
            if u != v:
                es.add((min(u, v), max(u, v)))
        stride *= L
    return n, sorted(es)


def random_edges(n, m, seed):
    rng = np.random.default_rng(seed)
    es = set()
    while len(es) < m:
        u, v = (int(x) for x in rng.integers(0, n, 2))
        if u != v:
            es.add((min(u, v), max(u, v)))
    return sorted(es)


def hub_edges(n, hub_degree, seed):
    """A hub joined to hub_degree sites, a ring through half of the rest, isolated sites."""
    rng = np.random.default_rng(seed)
    es = set((0, int(v)) for v in rng.choice(np.arange(1, n), hub_degree, replace=False))
    ring = list(range(n // 2, n - 3))
    for a, b in zip(ring, ring[1:] + ring[:1]):
        es.add((min(a, b), max(a, b)))
    return sorted(es)

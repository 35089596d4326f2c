"""Ising and Blume-Capel models on general graphs and sparse couplings over the C ABI.

Reference (paths inside MonteCarloX.jl):
  IsingGraph  (one J over a graph; no / uniform / per-site field)  SpinSystems/src/ising.jl:86-218
  IsingMatrix (symmetric sparse J_ij; same fields)                ising.jl:221-377
  Ising(graph, J; h), Ising(J::SparseMatrixCSC; h),
  Ising(graph, Jvec; h), Ising(dims; J, periodic, h)              ising.jl:383-428
  BlumeCapelGraph / BlumeCapelMatrix (crystal field D)           SpinSystems/src/blume_capel.jl:117-466
  BlumeCapel(graph, J, D; h), BlumeCapel(J, D; h), ...           blume_capel.jl:467-511

The reference takes its graphs from Graphs.jl (compat "1", not vendored); the parts it
uses are restated here from that package's published behaviour: a SimpleGraph is an
undirected graph without multi-edges whose neighbour lists are sorted; ``edges`` runs
over (u, v), u < v, in increasing u then v; ``grid(dims; periodic)`` numbers the site at
coordinates (x_1, ..., x_d) as x_1 + L_1 (x_2 + L_2 (...)) (first coordinate fastest)
and joins each site to its +-1 neighbours along every axis, wrapping around when
periodic (a ring of 2 is one edge, a ring of 1 none).  Indices are 0-based here.
"""
import ctypes as C

import numpy as np

from . import _lib as L
from . import (AbstractSpinSystem, ArgumentError, HeatBath, Philox, _check, default_context)

__all__ = ["SimpleGraph", "nv", "ne", "neighbors", "edges", "add_edge_", "grid", "IsingGraph", "IsingMatrix",
           "BlumeCapelGraph", "BlumeCapelMatrix", "GraphDevice", "IsingGraphDevice", "BlumeCapelGraphDevice",
           "delta_energy", "modify_", "graph_csr"]


class SimpleGraph:
    """Undirected simple graph on vertices 0..n-1 (Graphs.SimpleGraph)."""

    def __init__(self, n=0, edge_list=()):
        self._adj = [set() for _ in range(int(n))]
        for u, v in edge_list:
            add_edge_(self, u, v)

    def __repr__(self):
        return "SimpleGraph(nv=%d, ne=%d)" % (nv(self), ne(self))


def nv(g):
    return len(g._adj)


def ne(g):
    loops = sum(1 for v, a in enumerate(g._adj) if v in a)
    return (sum(len(a) for a in g._adj) - loops) // 2 + loops


def neighbors(g, v):
    return sorted(g._adj[v])


def add_edge_(g, u, v):
    u, v = int(u), int(v)
    if not (0 <= u < nv(g) and 0 <= v < nv(g)):
        raise ArgumentError("edge (%d, %d) outside 0..%d" % (u, v, nv(g) - 1))
    new = v not in g._adj[u]
    g._adj[u].add(v)
    g._adj[v].add(u)
    return new


def edges(g):
    """Edges (u, v) with u <= v, in increasing u, then v."""
    return [(u, v) for u in range(nv(g)) for v in sorted(g._adj[u]) if v >= u]


def grid(dims, periodic=False):
    """Graphs.grid(dims; periodic): hyper-cubic grid, first coordinate fastest."""
    dims = [int(d) for d in dims]
    n = int(np.prod(dims))
    g = SimpleGraph(n)
    stride = 1
    idx = np.arange(n, dtype=np.int64)
    for L_ in dims:
        x = (idx // stride) % L_
        if L_ > 1:
            fwd = np.where(x + 1 < L_, idx + stride, idx - (L_ - 1) * stride)
            ok = (x + 1 < L_) | periodic
            for u, v in zip(idx[ok], fwd[ok]):
                if u != v:
                    g._adj[int(u)].add(int(v))
                    g._adj[int(v)].add(int(u))
        stride *= L_
    return g


def graph_csr(g):
    """(rowptr int64[n+1], col int32[...]) with sorted rows."""
    rowptr = np.zeros(nv(g) + 1, np.int64)
    cols = []
    for v in range(nv(g)):
        nb = sorted(g._adj[v])
        cols.extend(nb)
        rowptr[v + 1] = rowptr[v] + len(nb)
    return rowptr, np.asarray(cols, np.int32)


def _field(h, n):
    if np.isscalar(h):
        return None, float(h)
    hv = np.ascontiguousarray(h, np.float64).reshape(-1)
    if hv.size != n:
        raise ArgumentError("Field vector length must match number of spins")
    return hv, 0.0


class GraphDevice(AbstractSpinSystem):
    """A spin system on a neighbour list held on the device (one coupling J when
    ``coupling`` is None, per-entry couplings otherwise).  All spins start at +1."""
    STATES = (-1, 1)
    MODEL = "Ising"
    D = 0.0

    def _create(self, hdl):
        _check(L.load().mcx_graph_create(
            self.ctx.handle, self.N, self.rowptr.ctypes.data, self.col.ctypes.data,
            None if self.coupling is None else self.coupling.ctypes.data,
            float(self.J) if self.coupling is None else 0.0,
            None if self.field is None else self.field.ctypes.data, self.h, C.byref(hdl)))

    def __init__(self, rowptr, col, coupling=None, J=1.0, h=0.0, ctx=None):
        self.ctx = ctx or default_context()
        self.rowptr = np.ascontiguousarray(rowptr, np.int64)
        self.col = np.ascontiguousarray(col, np.int32)
        self.N = len(self.rowptr) - 1
        self.coupling = None if coupling is None else np.ascontiguousarray(coupling, np.float64)
        if self.coupling is not None and self.coupling.size != self.col.size:
            raise ArgumentError("one coupling per stored entry expected")
        self.field, self.h = _field(h, self.N)
        self.J = float(J) if self.coupling is None else None
        hdl = C.c_void_p()
        self._create(hdl)
        self.handle = hdl

    @property
    def kind(self):
        return self.MODEL + ("Graph" if self.coupling is None else "Matrix")

    def __len__(self):
        return self.N

    @property
    def spins(self):
        out = np.empty(self.N, np.int8)
        _check(L.load().mcx_graph_get_spins(self.handle, out.ctypes.data, self.N))
        return out

    @spins.setter
    def spins(self, values):
        arr = np.ascontiguousarray(values, dtype=np.int8).reshape(-1)
        if arr.size != self.N:
            raise ArgumentError("expected %d spins, got %d" % (self.N, arr.size))
        _check(L.load().mcx_graph_set_spins(self.handle, arr.ctypes.data, self.N))

    @property
    def colours(self):
        """Colour class of every site (first-fit colouring in vertex order)."""
        out = np.empty(self.N, np.int32)
        _check(L.load().mcx_graph_colours(self.handle, out.ctypes.data, self.N))
        return out

    def info(self):
        n, c, e, b = C.c_int64(), C.c_int32(), C.c_int64(), C.c_int64()
        _check(L.load().mcx_graph_info(self.handle, C.byref(n), C.byref(c), C.byref(e), C.byref(b)))
        return {"sites": n.value, "colours": c.value, "entries": e.value, "device_bytes": b.value}

    def close(self):
        if getattr(self, "handle", None):
            L.load().mcx_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class IsingGraphDevice(GraphDevice):
    """IsingGraph / IsingMatrix on the device."""


class BlumeCapelGraphDevice(GraphDevice):
    """BlumeCapelGraph / BlumeCapelMatrix on the device (spins in {-1, 0, 1})."""
    STATES = (-1, 0, 1)
    MODEL = "BlumeCapel"

    def __init__(self, rowptr, col, coupling=None, J=1.0, D=0.0, h=0.0, ctx=None):
        self.D = float(D)
        super().__init__(rowptr, col, coupling, J=J, h=h, ctx=ctx)

    def _create(self, hdl):
        _check(L.load().mcx_bcgraph_create(
            self.ctx.handle, self.N, self.rowptr.ctypes.data, self.col.ctypes.data,
            None if self.coupling is None else self.coupling.ctypes.data,
            float(self.J) if self.coupling is None else 0.0, self.D,
            None if self.field is None else self.field.ctypes.data, self.h, C.byref(hdl)))


def IsingGraph(graph, J=1, *, h=0, ctx=None):
    """IsingGraph(graph, J; h) (ising.jl:117-139); self-loops are not supported."""
    if any(v in graph._adj[v] for v in range(nv(graph))):
        raise ArgumentError("self-loops are not supported")
    rowptr, col = graph_csr(graph)
    return IsingGraphDevice(rowptr, col, None, J=J, h=h, ctx=ctx)


def _csr(J):
    import scipy.sparse as sp
    A = J if sp.issparse(J) else sp.csr_matrix(np.asarray(J, np.float64))
    if A.shape[0] != A.shape[1]:
        raise ArgumentError("Sparse J must be square")
    A = sp.csr_matrix(A, dtype=np.float64)
    A.sum_duplicates()
    A.sort_indices()
    return A.indptr.astype(np.int64), A.indices.astype(np.int32), A.data


def IsingMatrix(J, *, h=0, ctx=None):
    """IsingMatrix(J::SparseMatrixCSC; h) (ising.jl:265-292): a square symmetric scipy
    sparse matrix or a dense 2-D array; diagonal entries are ignored."""
    rp, col, val = _csr(J)
    return IsingGraphDevice(rp, col, val, h=h, ctx=ctx)


def BlumeCapelGraph(graph, J=1, D=0, *, h=0, ctx=None):
    """BlumeCapelGraph(graph, J, D; h) (blume_capel.jl:154-190)."""
    if any(v in graph._adj[v] for v in range(nv(graph))):
        raise ArgumentError("self-loops are not supported")
    rowptr, col = graph_csr(graph)
    return BlumeCapelGraphDevice(rowptr, col, None, J=J, D=D, h=h, ctx=ctx)


def BlumeCapelMatrix(J, D=0, *, h=0, ctx=None):
    """BlumeCapelMatrix(J::SparseMatrixCSC, D; h) (blume_capel.jl:328-360)."""
    rp, col, val = _csr(J)
    return BlumeCapelGraphDevice(rp, col, val, D=D, h=h, ctx=ctx)


def matrix_from_edges(graph, Jvec):
    """The symmetric coupling matrix of Ising(graph, Jvec) (ising.jl:391-411): J[k] on
    the k-th edge of edges(graph)."""
    import scipy.sparse as sp
    E = edges(graph)
    Jvec = np.asarray(Jvec, np.float64).reshape(-1)
    if len(E) != Jvec.size:
        raise ArgumentError("Length of J vector must equal number of graph edges")
    if not E:
        return sp.csr_matrix((nv(graph), nv(graph)))
    u = np.array([e[0] for e in E] + [e[1] for e in E])
    v = np.array([e[1] for e in E] + [e[0] for e in E])
    return sp.csr_matrix((np.concatenate([Jvec, Jvec]), (u, v)), shape=(nv(graph), nv(graph)))


def delta_energy(sys, i, s_new=None):
    """delta_energy(sys, i) of a flip (Ising, ising.jl:20-23) or delta_energy(sys, i, s_new)
    (blume_capel.jl:32-35); 0-based site."""
    out = C.c_double()
    if s_new is None:
        _check(L.load().mcx_graph_delta_energy(sys.handle, int(i), C.byref(out)))
    else:
        _check(L.load().mcx_graph_delta_energy_to(sys.handle, int(i), int(s_new), C.byref(out)))
    return out.value


def modify_(sys, i, s_new=None):
    """modify!(sys, i, ...): flip site i (Ising) or set it to s_new, updating the cache."""
    if s_new is None:
        _check(L.load().mcx_graph_flip(sys.handle, int(i)))
    else:
        _check(L.load().mcx_graph_set_site(sys.handle, int(i), int(s_new)))
    return sys


def spin_flip(sys, alg, n=1):
    """n x spin_flip!(sys, alg) at uniformly random vertices, in order, with the reference's
    FP64 rule (mcx_graph_spin_flip); advances alg.rng and the counters like sweep."""
    rng = alg.rng._c()
    cnt = L.mcx_counters(0, 0)
    _check(L.load().mcx_graph_spin_flip(sys.handle, alg.ALG, float(alg.beta), C.byref(rng), int(n), C.byref(cnt)))
    alg.rng.counter = rng.counter
    alg.steps += cnt.attempts
    if isinstance(alg, HeatBath):
        alg.flips += cnt.accepted
    else:
        alg.accepted += cnt.accepted


def sweep(sys, alg, nsweeps=1, record=False):
    beta = alg.beta
    rng = alg.rng._c()
    cnt = L.mcx_counters(0, 0)
    Es = np.zeros(nsweeps, np.float64) if record else None
    Ms = np.zeros(nsweeps, np.int64) if record else None
    _check(L.load().mcx_graph_sweep(sys.handle, alg.ALG, float(beta), C.byref(rng), int(nsweeps),
                                    Es.ctypes.data if record else None, Ms.ctypes.data if record else None,
                                    C.byref(cnt)))
    alg.rng.counter = rng.counter
    alg.steps += cnt.attempts
    if isinstance(alg, HeatBath):
        alg.flips += cnt.accepted
    else:
        alg.accepted += cnt.accepted
    return (Es, Ms) if record else None


def energy(sys, full=False):
    E, M = C.c_double(), C.c_int64()
    _check(L.load().mcx_graph_energy(sys.handle, 1 if full else 0, C.byref(E), C.byref(M)))
    return E.value, M.value


def init(sys, t, rng=None):
    if t == "random":
        r = rng if isinstance(rng, Philox) else Philox(rng)
        _check(L.load().mcx_graph_init_random(sys.handle, r.seed, r.stream))
    else:
        _check(L.load().mcx_graph_init_uniform(sys.handle, {"up": 1, "down": -1, "zero": 0}[t]))

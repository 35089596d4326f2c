"""Batched parallel tempering on the device (ParallelTempering / ReplicaExchange mirror).

Reference (paths inside MonteCarloX.jl):
  ParallelTempering(betas; seed, rng)   src/algorithms/parallel_tempering.jl:24-53
  set_betas(n, bmin, bmax, mode)        src/algorithms/parallel_tempering.jl:146-162
  update!(rx, xs) / index / steps / accepted / acceptance_rate(s)
                                        src/algorithms/replica_exchange.jl:13-178
Several independent ladders (e.g. one per lattice size) live in one object; every
ladder behaves as its own ReplicaExchange, and all of them are swept and exchanged
together on the GPU.
"""
import ctypes as C
from fractions import Fraction
import math

import numpy as np

from . import _lib as L
from . import _check, default_context, Philox, ArgumentError

__all__ = ["set_betas", "ParallelTempering"]


def set_betas(nreplicas, bmin, bmax, mode, T=float):
    """Beta ladder from bmax down to bmin, `:uniform` or `:geometric`
    (parallel_tempering.jl:146-162).  Points are the correctly rounded values of the
    exact range, as Julia's range() gives them."""
    mode = mode.lstrip(":") if isinstance(mode, str) else mode
    n = int(nreplicas)
    if n < 2:
        raise ArgumentError("nreplicas must be >= 2")

    def rng(a, b):
        fa, fb = Fraction(a), Fraction(b)
        return [float(fa + (fb - fa) * i / (n - 1)) for i in range(n)]

    if mode == "uniform":
        vals = rng(float(bmax), float(bmin))
    elif mode == "geometric":
        vals = [math.exp(v) for v in rng(math.log(float(bmax)), math.log(float(bmin)))]
    else:
        raise ArgumentError("unknown beta mode %s; use :uniform or :geometric" % mode)
    return [T(v) for v in vals]


_ALG = {"metropolis": L.METROPOLIS, "glauber": L.GLAUBER, "heatbath": L.HEATBATH}


class ParallelTempering:
    """Ladders of Ising replicas on the device.

    ladders: list of (L, betas) -- one ladder per lattice side L, betas by ladder
    position (position 0 first, as set_betas returns them)."""

    def __init__(self, ladders, *, dim=3, J=1, h=0, seed=1000, ctx=None):
        self.ctx = ctx or default_context()
        self.dim = int(dim)
        self.J, self.h = J, h
        self.sides = [int(l) for l, _ in ladders]
        self.ladder_betas = [list(map(float, b)) for _, b in ladders]
        self.sizes = [len(b) for b in self.ladder_betas]
        betas = np.array([b for bs in self.ladder_betas for b in bs], np.float64)
        sides = (C.c_int32 * len(self.sides))(*self.sides)
        ns = (C.c_int32 * len(self.sizes))(*self.sizes)
        h_ = C.c_void_p()
        _check(L.load().mcx_pt_create(self.ctx.handle, self.dim, len(self.sides), sides, ns,
                                      betas.ctypes.data_as(C.POINTER(C.c_double)), float(J), float(h), C.byref(h_)))
        self.handle = h_
        self.nrep = int(sum(self.sizes))
        self.npos = self.nrep  # one replica per ladder position
        self.rng = Philox(seed)
        self.replica_ladder = [l for l, n in enumerate(self.sizes) for _ in range(n)]
        self._record = "request"

    # -- series and autocorrelation times -------------------------------------
    def record_(self, mode):
        """Which series sweep_ keeps on the device: "request" (only with record=True, per
        replica), "replica" (always, per replica) or "position" (always, one column per
        global ladder position: the trace at each fixed beta)."""
        code = {"request": 0, "replica": 1, "position": 2}[mode]
        _check(L.load().mcx_pt_set_record(self.handle, code))
        self._record = mode
        return self

    def tau_int(self, quantity="energy", *, min_points=2, max_lag=None, c=5.0, by=None):
        """integrated_autocorrelation_times of the columns of the last run's device series
        (src/measurements/autocorrelations.jl:69-102); ``by`` ("replica" / "position")
        checks which columns the series holds."""
        if by is not None and (by == "position") != (self._record == "position"):
            raise ArgumentError("the device series is kept by %s; call record_(%r) before the run"
                                % ("position" if self._record == "position" else "replica", by))
        taus = np.empty(self.nrep, np.float64)
        _check(L.load().mcx_pt_tau_int(self.handle, {"energy": 0, "magnetization": 1}[quantity], int(min_points),
                                       0 if max_lag is None else int(max_lag), float(c), taus.ctypes.data))
        return taus

    # -- state ---------------------------------------------------------------
    def init_(self, seed):
        _check(L.load().mcx_pt_init_random(self.handle, int(seed)))

    def nsites(self, r):
        return self.sides[self.replica_ladder[r]] ** self.dim

    def spins(self, r):
        out = np.empty(self.nsites(r), np.int8)
        _check(L.load().mcx_pt_get_spins(self.handle, int(r), out.ctypes.data, out.size))
        return out

    def set_spins_(self, r, values):
        arr = np.ascontiguousarray(values, np.int8).reshape(-1)
        _check(L.load().mcx_pt_set_spins(self.handle, int(r), arr.ctypes.data, arr.size))

    def observables(self):
        P = np.empty(self.nrep, np.int64)
        M = np.empty(self.nrep, np.int64)
        _check(L.load().mcx_pt_observables(self.handle, P.ctypes.data, M.ctypes.data))
        return P, M

    def energies(self):
        P, M = self.observables()
        return (-(self.J * P.astype(np.float64))) - (self.h * M.astype(np.float64))

    @property
    def positions(self):
        """0-based ladder position of each replica (rx.indices - 1)."""
        pos = np.empty(self.nrep, np.int32)
        st = C.c_int32()
        _check(L.load().mcx_pt_indices(self.handle, pos.ctypes.data, C.byref(st)))
        return pos

    @property
    def indices(self):
        """rx.indices: 1-based ladder position of each replica (replica_exchange.jl:48-50)."""
        return self.positions + 1

    @property
    def stage(self):
        st = C.c_int32()
        _check(L.load().mcx_pt_indices(self.handle, None, C.byref(st)))
        return st.value

    def betas_of_replicas(self):
        pos = self.positions
        return np.array([self.ladder_betas[self.replica_ladder[r]][pos[r]] for r in range(self.nrep)])

    def counters(self):
        """(steps, accepted) per ladder edge, ladder after ladder."""
        ne = sum(n - 1 for n in self.sizes)
        s = np.empty(ne, np.uint64)
        a = np.empty(ne, np.uint64)
        _check(L.load().mcx_pt_exchange_counters(self.handle, s.ctypes.data, a.ctypes.data))
        return s, a

    def acceptance_rates(self):
        s, a = self.counters()
        return np.where(s > 0, a / np.maximum(s, 1), 0.0)

    def acceptance_rate(self):
        s, a = self.counters()
        return float(a.sum() / s.sum()) if s.sum() > 0 else 0.0

    # -- running -------------------------------------------------------------
    def sweep_(self, nsweeps, alg="metropolis", exchange_every=1, mode="persistent", record=False):
        """`nsweeps` sweeps of every replica with an exchange step after every
        `exchange_every`-th sweep.  Returns the (nsweeps, nrep, 2) series of
        (pair_sum, spin_sum) if `record` (columns by replica, or by global ladder position
        after record_("position"))."""
        rng = self.rng._c()
        out = np.empty((nsweeps, self.nrep, 2), np.int64) if record else None
        m = {"persistent": L.PT_PERSISTENT, "plain": L.PT_PLAIN}[mode]
        _check(L.load().mcx_pt_run(self.handle, _ALG[alg], C.byref(rng), int(nsweeps), int(exchange_every), m,
                                   out.ctypes.data if record else None))
        self.rng.counter = rng.counter
        return out

    # -- schedule of the persistent form (results never depend on it) ------------
    def set_schedule(self, blocks_per_sm=0, vcap=16, weights=0):
        """Blocks per SM (0 = the co-resident maximum), the widest chunk of sites per thread
        (16, 8 or 4) and the warp-split cost weights (0, 1, 2) of the persistent kernel."""
        _check(L.load().mcx_pt_set_schedule(self.handle, int(blocks_per_sm), int(vcap), int(weights)))

    @property
    def schedule(self):
        """(blocks_per_sm, vcap, weights, max_blocks_per_sm)."""
        v = [C.c_int32() for _ in range(4)]
        _check(L.load().mcx_pt_get_schedule(self.handle, *[C.byref(x) for x in v]))
        return tuple(x.value for x in v)

    def autotune_(self, alg="metropolis", exchange_every=1, sweeps=20):
        """Time every schedule on the ladder's own state (restored afterwards) and keep the
        fastest; returns (blocks_per_sm, vcap, weights, ns per attempt)."""
        b, v, w = C.c_int32(), C.c_int32(), C.c_int32()
        ns = C.c_double()
        _check(L.load().mcx_pt_autotune(self.handle, _ALG[alg], int(exchange_every), int(sweeps), C.byref(b),
                                        C.byref(v), C.byref(w), C.byref(ns)))
        return b.value, v.value, w.value, ns.value

    def set_wait_limit(self, polls):
        _check(L.load().mcx_pt_set_wait_limit(self.handle, int(polls)))

    def close(self):
        if getattr(self, "handle", None):
            L.load().mcx_pt_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

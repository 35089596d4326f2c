"""Host-side mirror of the MonteCarloX.jl / SpinSystems API for the GB300 path.

Every compute call goes through the C ABI of ``libmcx_cuda.so`` (``include/mcx.h``);
there is no CPU fallback.  Names follow the reference with Julia's ``!`` written as
a trailing underscore (``init!`` -> ``init_``, ``spin_flip!`` -> ``spin_flip_``).

Reference API mirrored here (paths inside MonteCarloX.jl):
  BoltzmannEnsemble           src/ensembles/boltzmann.jl:7-30
  Metropolis / Glauber        src/algorithms/metropolis.jl:63-127
  HeatBath                    src/algorithms/heat_bath.jl:11-17
  acceptance_rate / reset!    src/algorithms/importance_sampling.jl:95-110
  Ising / IsingLatticeOptim   SpinSystems/src/ising.jl:413-461
  IsingGraph / IsingMatrix    SpinSystems/src/ising.jl:86-428 (mcx.graph)
  BlumeCapel                  SpinSystems/src/blume_capel.jl:500-511
  init! / energy / magnetization  ising.jl:17-18, :60-78, blume_capel.jl:18-19, :87-109
"""
import ctypes as C
import math

import numpy as np

from . import _lib as L

__all__ = [
    "MCXError", "ArgumentError", "BoundsError", "OutOfMemoryError", "BudgetError", "DeviceTimeoutError",
    "CudaError", "Context", "default_context", "Philox", "BoltzmannEnsemble", "logweight", "Metropolis",
    "Glauber", "HeatBath", "ensemble", "acceptance_rate", "reset_", "AbstractSystem", "AbstractSpinSystem",
    "Ising", "IsingLatticeOptim", "BlumeCapel", "init_", "energy", "magnetization", "observables",
    "sweep_", "spin_flip_", "set_spins_", "logistic", "autotune_",
]


# --------------------------------------------------------------------- errors --
class MCXError(RuntimeError):
    status = None


class ArgumentError(MCXError, ValueError):
    status = L.MCX_ERR_INVALID_ARG


class BoundsError(MCXError, IndexError):
    """An energy left the histogram range (the reference's BoundsError)."""
    status = L.MCX_ERR_OUT_OF_RANGE


class OutOfMemoryError(MCXError, MemoryError):
    status = L.MCX_ERR_OOM


class BudgetError(MCXError):
    status = L.MCX_ERR_BUDGET


class DeviceTimeoutError(MCXError, TimeoutError):
    status = L.MCX_ERR_TIMEOUT


class CudaError(MCXError):
    status = L.MCX_ERR_CUDA


class NotReadyError(MCXError):
    status = L.MCX_ERR_NOT_READY


class NotFoundError(MCXError, KeyError):
    status = L.MCX_ERR_NOT_FOUND


_ERRORS = {e.status: e for e in (ArgumentError, BoundsError, OutOfMemoryError, BudgetError,
                                 DeviceTimeoutError, CudaError, NotReadyError, NotFoundError)}


def _check(status):
    if status != L.MCX_OK:
        raise _ERRORS.get(status, MCXError)("%s: %s" % (L.load().mcx_status_string(status).decode(),
                                                        L.error_string()))


# -------------------------------------------------------------------- context --
class Context:
    """One CUDA stream plus the device memory owned through it (mcx_ctx)."""

    def __init__(self, device=0, stream=None, hbm_budget=0):
        lib = L.load()
        cfg = L.mcx_config(int(device), C.c_void_p(int(stream) if stream else 0), int(hbm_budget))
        h = C.c_void_p()
        _check(lib.mcx_ctx_create(C.byref(cfg), C.byref(h)))
        self.handle = h
        self.device = device

    def sync(self):
        _check(L.load().mcx_sync(self.handle))

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        _check(L.load().mcx_ctx_stream(self.handle, C.byref(s)))
        return s.value or 0

    def memory(self):
        used, budget = C.c_uint64(), C.c_uint64()
        _check(L.load().mcx_ctx_memory(self.handle, C.byref(used), C.byref(budget)))
        return used.value, budget.value

    def launches(self) -> int:
        n = C.c_uint64()
        _check(L.load().mcx_ctx_launches(self.handle, C.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "handle", None):
            L.load().mcx_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context()
    return _default_ctx


# ------------------------------------------------------------------------ rng --
class Philox:
    """Counter-based Philox4x32-10 stream: (seed, stream) key, counter = next sweep.

    Plays the role of the ``rng`` objects (Xoshiro / MersenneTwister) the reference
    algorithms carry; the counter advances by the number of sweeps run, so a run
    can be resumed or replayed exactly."""

    def __init__(self, seed=0, stream=0, counter=0):
        self.seed = int(seed) & (2 ** 64 - 1)
        self.stream = int(stream) & 0xFFFFFFFF
        self.counter = int(counter)

    def _c(self):
        return L.mcx_rng(self.seed, self.counter, self.stream, 0)

    def __repr__(self):
        return "Philox(seed=%d, stream=%d, counter=%d)" % (self.seed, self.stream, self.counter)


# ------------------------------------------------------------------ ensembles --
def logistic(x):
    """src/infrastructure/utils.jl:82-88"""
    if x >= 0:
        return 1.0 / (1.0 + math.exp(-x))
    ex = math.exp(x)
    return ex / (1.0 + ex)


class BoltzmannEnsemble:
    """logweight(E) = -beta*E; exactly one of beta / β / T (src/ensembles/boltzmann.jl:7-22)."""

    def __init__(self, *, beta=None, T=None, **kw):
        b2 = kw.pop("β", None)
        if kw:
            raise TypeError("unexpected keyword(s) %s" % list(kw))
        if beta is not None and b2 is not None:
            raise ArgumentError("Specify only one of `beta` or `β`")
        b = beta if beta is not None else b2
        if (b is None) == (T is None):
            raise ArgumentError("Specify exactly one of `beta`/`β` or `T`")
        self.beta = b if b is not None else 1.0 / T

    def logweight(self, E):
        return -self.beta * E

    def __call__(self, E):
        return self.logweight(E)

    def __eq__(self, other):
        return type(other) is type(self) and other.beta == self.beta


def logweight(ens, x=None):
    f = ens.logweight if hasattr(ens, "logweight") else ens
    return f if x is None else f(x)


# ----------------------------------------------------------------- algorithms --
class _ImportanceSampling:
    ALG = None

    def __init__(self, rng, ensemble=None, *, beta=None, **kw):
        b2 = kw.pop("β", None)
        if kw:
            raise TypeError("unexpected keyword(s) %s" % list(kw))
        if ensemble is None:
            if beta is None and b2 is None:
                raise ArgumentError("give an ensemble or beta")
            ensemble = BoltzmannEnsemble(beta=beta if beta is not None else b2)
        self.rng = rng if isinstance(rng, Philox) else Philox(rng)
        self.ensemble = ensemble
        self.steps = 0
        self.accepted = 0

    @property
    def beta(self):
        return self.ensemble.beta


class Metropolis(_ImportanceSampling):
    """Metropolis(rng; β) -- accept iff lr > 0 || U < exp(lr)."""
    ALG = L.METROPOLIS


class Glauber(_ImportanceSampling):
    """Glauber(rng; β) -- accept iff U < logistic(lr)."""
    ALG = L.GLAUBER


class HeatBath:
    """HeatBath(rng; β): fields rng, β (as ``beta``), steps (src/algorithms/heat_bath.jl:11-17).

    ``flips`` counts state changes, which the reference does not keep."""
    ALG = L.HEATBATH

    def __init__(self, rng, *, beta=None, **kw):
        b2 = kw.pop("β", None)
        if kw:
            raise TypeError("unexpected keyword(s) %s" % list(kw))
        b = beta if beta is not None else b2
        if b is None:
            raise ArgumentError("HeatBath needs β")
        self.rng = rng if isinstance(rng, Philox) else Philox(rng)
        self.beta = b
        self.steps = 0
        self.flips = 0


def ensemble(alg):
    return alg.ensemble


def acceptance_rate(alg):
    """accepted/steps, 0.0 before the first step (importance_sampling.jl:95-96)."""
    return alg.accepted / alg.steps if alg.steps > 0 else 0.0


def reset_(alg):
    """Zero the step / acceptance counters (importance_sampling.jl:106-110)."""
    alg.steps = 0
    if hasattr(alg, "accepted"):
        alg.accepted = 0
    if hasattr(alg, "flips"):
        alg.flips = 0
    if hasattr(alg, "_reset_hook"):
        alg._reset_hook()


# -------------------------------------------------------------------- systems --
class AbstractSystem:
    pass


class AbstractSpinSystem(AbstractSystem):
    pass


class DeviceLattice(AbstractSpinSystem):
    MODEL = None
    STATES = ()

    def __init__(self, dims, *, J=1, D=0, h=0, periodic=True, layout="int8", ctx=None):
        if not periodic:
            raise ArgumentError("the device lattices are periodic")
        if not isinstance(h, (int, float)):
            raise ArgumentError("the device lattices take a uniform field h")
        self.ctx = ctx or default_context()
        self.dims = [int(d) for d in dims]
        self.J, self.D, self.h = J, D, h
        self.layout = layout
        lay = {"int8": L.LAYOUT_INT8, "msc64": L.LAYOUT_MSC64}[layout]
        Ls = (C.c_int32 * 3)(*(self.dims + [1] * (3 - len(self.dims))))
        hdl = C.c_void_p()
        _check(L.load().mcx_lattice_create(self.ctx.handle, self.MODEL, len(self.dims), Ls, lay, float(J),
                                           float(D), float(h), C.byref(hdl)))
        self.handle = hdl
        self.N = int(np.prod(self.dims))
        self.uniforms = "site"

    def __len__(self):
        return self.N

    def set_uniforms(self, form="planes"):
        """How the sweeps of this lattice draw their uniforms (mcx_lattice_set_uniforms):
        "site" (one Philox word per site, the default) or "planes" (Ising, Lx a multiple of
        128: bit planes for the top 8 bits of every uniform, compared for 64 sites at once;
        Blume-Capel: bit planes for the proposal bits).  Same distribution, different chain."""
        _check(L.load().mcx_lattice_set_uniforms(self.handle, {"site": 0, "planes": 1}[form]))
        self.uniforms = form

    def set_packing(self, allow=True):
        """Whether multi-sweep calls may run on a transient 64-sites-per-word copy of this
        int8 Ising lattice (mcx_lattice_set_packing; results are identical either way)."""
        _check(L.load().mcx_lattice_set_packing(self.handle, 1 if allow else 0))

    @property
    def spins(self):
        """Copy of the spins in SpinSystems linear order (int8)."""
        out = np.empty(self.N, np.int8)
        _check(L.load().mcx_get_spins(self.handle, out.ctypes.data, self.N))
        return out

    @spins.setter
    def spins(self, values):
        set_spins_(self, values)

    def close(self):
        if getattr(self, "handle", None):
            L.load().mcx_lattice_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class IsingDevice(DeviceLattice):
    MODEL = L.ISING
    STATES = (-1, 1)


class BlumeCapelDevice(DeviceLattice):
    MODEL = L.BLUME_CAPEL
    STATES = (-1, 0, 1)


def _lattice_ok(dims):
    return len(dims) in (2, 3) and all(isinstance(d, (int, np.integer)) and d >= 4 and d % 2 == 0 for d in dims)


def Ising(dims, J=None, *, periodic=True, h=0, layout="int8", ctx=None):
    """The reference's Ising constructors (SpinSystems/src/ising.jl:383-428), all spins up.

    * ``Ising(dims; J=1, periodic=true, h=0)`` with a scalar J and h on an even periodic
      2-D / 3-D grid (every side >= 4): the colour-split device lattice.
    * Other grids (open boundaries, odd or short sides, 1-D or >3-D), a field vector
      ``h``, or a coupling vector ``J`` over the grid's edges: the general-graph system
      on ``grid(dims; periodic)``.
    * ``Ising(graph::SimpleGraph, J::Real; h)``: IsingGraph; ``Ising(graph, Jvec; h)``:
      IsingMatrix with Jvec on edges(graph); ``Ising(J::sparse; h)``: IsingMatrix."""
    from . import graph as G
    if isinstance(dims, G.SimpleGraph):
        if J is None or np.isscalar(J):
            return G.IsingGraph(dims, 1 if J is None else J, h=h, ctx=ctx)
        return G.IsingMatrix(G.matrix_from_edges(dims, J), h=h, ctx=ctx)
    if J is None and not isinstance(dims, (list, tuple, np.ndarray)):
        return G.IsingMatrix(dims, h=h, ctx=ctx)  # Ising(J::SparseMatrixCSC; h)
    J = 1 if J is None else J
    dims = [int(d) for d in dims]
    if np.isscalar(J) and np.isscalar(h) and periodic and _lattice_ok(dims):
        return IsingDevice(dims, J=J, h=h, periodic=periodic, layout=layout, ctx=ctx)
    if layout != "int8":
        raise ArgumentError("layout %r needs an even periodic 2-D / 3-D grid with a scalar J and h" % layout)
    g = G.grid(dims, periodic=periodic)
    if np.isscalar(J):
        return G.IsingGraph(g, J, h=h, ctx=ctx)
    import scipy.sparse as sp
    if sp.issparse(J):
        return G.IsingMatrix(J, h=h, ctx=ctx)
    return G.IsingMatrix(G.matrix_from_edges(g, J), h=h, ctx=ctx)


def IsingLatticeOptim(Lx, Ly, *, layout="int8", ctx=None):
    """2-D periodic J=1 Ising (SpinSystems/src/ising.jl:430-461)."""
    return IsingDevice([Lx, Ly], J=1, h=0, layout=layout, ctx=ctx)


def BlumeCapel(dims, J=None, D=0, *, periodic=True, h=0, ctx=None):
    """The reference's BlumeCapel constructors (SpinSystems/src/blume_capel.jl:467-511), all
    spins up: ``BlumeCapel(dims; J=1, D=0, periodic=true, h=0)`` on the colour-split lattice
    for a scalar J and h on an even periodic 2-D / 3-D grid (every side >= 4), otherwise on
    the general-graph path; ``BlumeCapel(graph, J, D; h)``, ``BlumeCapel(graph, Jvec, D; h)``
    and ``BlumeCapel(J::sparse, D; h)``."""
    from . import graph as G
    if isinstance(dims, G.SimpleGraph):
        if J is None or np.isscalar(J):
            return G.BlumeCapelGraph(dims, 1 if J is None else J, D, h=h, ctx=ctx)
        return G.BlumeCapelMatrix(G.matrix_from_edges(dims, J), D, h=h, ctx=ctx)
    if not isinstance(dims, (list, tuple, np.ndarray)):
        return G.BlumeCapelMatrix(dims, 0 if J is None else J, h=h, ctx=ctx)  # BlumeCapel(J::sparse, D; h)
    J = 1 if J is None else J
    dims = [int(d) for d in dims]
    if np.isscalar(J) and np.isscalar(h) and periodic and _lattice_ok(dims):
        return BlumeCapelDevice(dims, J=J, D=D, h=h, periodic=periodic, ctx=ctx)
    g = G.grid(dims, periodic=periodic)
    if np.isscalar(J):
        return G.BlumeCapelGraph(g, J, D, h=h, ctx=ctx)
    import scipy.sparse as sp
    if sp.issparse(J):
        return G.BlumeCapelMatrix(J, D, h=h, ctx=ctx)
    return G.BlumeCapelMatrix(G.matrix_from_edges(g, J), D, h=h, ctx=ctx)


def _is_graph(sys):
    from .graph import GraphDevice
    return isinstance(sys, GraphDevice)


def set_spins_(sys, values):
    if _is_graph(sys):
        sys.spins = values
        return
    arr = np.ascontiguousarray(values, dtype=np.int8).reshape(-1)
    if arr.size != sys.N:
        raise ArgumentError("expected %d spins, got %d" % (sys.N, arr.size))
    _check(L.load().mcx_set_spins(sys.handle, arr.ctypes.data, sys.N))


def init_(sys, type, rng=None):
    """init!(sys, :up | :down | :zero | :random; rng)."""
    t = type.lstrip(":") if isinstance(type, str) else type
    if _is_graph(sys):
        from . import graph as G
        if t == "random" and rng is None:
            raise ArgumentError("Random initialization requires rng")
        if t not in ("random", "up", "down", "zero") or (t == "zero" and 0 not in sys.STATES):
            raise ArgumentError("Unknown initialization type: %s" % type)
        G.init(sys, t, rng)
        return sys
    if t == "random":
        if rng is None:
            raise ArgumentError("Random initialization requires rng")
        r = rng if isinstance(rng, Philox) else Philox(rng)
        _check(L.load().mcx_init_random(sys.handle, r.seed, r.stream))
    elif t in ("up", "down", "zero"):
        v = {"up": 1, "down": -1, "zero": 0}[t]
        if v not in sys.STATES:
            raise ArgumentError("Unknown initialization type: %s" % type)
        _check(L.load().mcx_init_uniform(sys.handle, v))
    else:
        raise ArgumentError("Unknown initialization type: %s" % type)
    return sys


def observables(sys, full=False):
    """(pair_sum, spin_sum, spin2_sum); ``full=True`` recomputes them from the spins."""
    P, M, Q = C.c_int64(), C.c_int64(), C.c_int64()
    fn = L.load().mcx_recompute_observables if full else L.load().mcx_observables
    _check(fn(sys.handle, C.byref(P), C.byref(M), C.byref(Q)))
    return P.value, M.value, Q.value


def energy(sys, full=False):
    """energy(sys; full): -J*pair - h*M (+ D*sum s^2 for Blume-Capel); -pair - field on a
    general graph."""
    if _is_graph(sys):
        from . import graph as G
        return G.energy(sys, full)[0]
    P, M, Q = observables(sys, full)
    E = (-(sys.J * P)) - (sys.h * M)
    if isinstance(sys, BlumeCapelDevice):
        E = E + sys.D * Q
    return E


def magnetization(sys, full=False):
    if _is_graph(sys):
        from . import graph as G
        return G.energy(sys, full)[1]
    return observables(sys, full)[1]


def sweep_(sys, alg, nsweeps=1, record=False):
    """``nsweeps`` checkerboard sweeps (N spin_flip! attempts each) on the device.

    Updates ``alg.steps`` / ``alg.accepted`` (HeatBath: ``steps``, ``flips``) and the
    rng counter.  With ``record=True`` returns the per-sweep (pair, spin, spin2) series
    as an int64 array of shape (nsweeps, 3); on a general graph, colour-class sweeps
    returning (E float64[nsweeps], M int64[nsweeps])."""
    if _is_graph(sys):
        from . import graph as G
        return G.sweep(sys, alg, nsweeps, record)
    beta = alg.beta
    rng = alg.rng._c()
    cnt = L.mcx_counters(0, 0)
    obs = np.zeros((nsweeps, 3), np.int64) if record else None
    _check(L.load().mcx_sweep(sys.handle, alg.ALG, float(beta), C.byref(rng), int(nsweeps),
                              obs.ctypes.data if record else None, C.byref(cnt)))
    alg.rng.counter = rng.counter
    alg.steps += cnt.attempts
    if isinstance(alg, HeatBath):
        alg.flips += cnt.accepted
    else:
        alg.accepted += cnt.accepted
    return obs


def sweep_batch_(systems, algs, nsweeps=1, record=False):
    """``nsweeps`` sweeps of every lattice systems[i] with algs[i] (one algorithm kind,
    each with its own beta and rng), as one device call: the independent chains of the
    reference's ParallelChains (src/infrastructure/parallel_chains.jl).  Results are those
    of sweep_(systems[i], algs[i], nsweeps) bit for bit; returns the per-sweep series of
    every lattice when ``record``."""
    n = len(systems)
    if n != len(algs) or n == 0:
        raise ArgumentError("one algorithm per system, at least one")
    kinds = {a.ALG for a in algs}
    if len(kinds) != 1:
        raise ArgumentError("a batch runs one algorithm kind")
    handles = (C.c_void_p * n)(*[s.handle.value if isinstance(s.handle, C.c_void_p) else s.handle for s in systems])
    betas = np.array([float(a.beta) for a in algs], np.float64)
    rngs = (L.mcx_rng * n)(*[a.rng._c() for a in algs])
    cnts = (L.mcx_counters * n)()
    obs = [np.zeros((nsweeps, 3), np.int64) for _ in range(n)] if record else None
    ptrs = (C.c_void_p * n)(*[o.ctypes.data for o in obs]) if record else None
    _check(L.load().mcx_sweep_batch(handles, n, algs[0].ALG, betas.ctypes.data_as(C.POINTER(C.c_double)), rngs,
                                    int(nsweeps), ptrs, cnts))
    for i, a in enumerate(algs):
        a.rng.counter = rngs[i].counter
        a.steps += cnts[i].attempts
        if isinstance(a, HeatBath):
            a.flips += cnts[i].accepted
        else:
            a.accepted += cnts[i].accepted
    return obs


def autotune_(sys, alg):
    """Pick the fastest kernel shape for this lattice and algorithm (results unchanged).
    Returns (sites per thread, ns per site per half-sweep)."""
    v = C.c_int32()
    ns = C.c_double()
    _check(L.load().mcx_autotune(sys.handle, alg.ALG, float(alg.beta), C.byref(v), C.byref(ns)))
    return v.value, ns.value


def spin_flip_(sys, alg, n=1):
    """spin_flip!(sys, alg) (SpinSystems/src/ising.jl:25-58, blume_capel.jl:41-85), ``n``
    times: single-site updates at uniformly random sites in the reference's own order and
    with its FP64 decisions, run on the device one after another.  Advances ``alg.rng`` by
    ``n`` and the algorithm's counters like ``sweep_``.  A loop written around spin_flip!
    runs unchanged; ``sweep_`` is the fast path."""
    if _is_graph(sys):
        from . import graph as G
        return G.spin_flip(sys, alg, n)
    rng = alg.rng._c()
    cnt = L.mcx_counters(0, 0)
    _check(L.load().mcx_spin_flip(sys.handle, alg.ALG, float(alg.beta), C.byref(rng), int(n), C.byref(cnt)))
    alg.rng.counter = rng.counter
    alg.steps += cnt.attempts
    if isinstance(alg, HeatBath):
        alg.flips += cnt.accepted
    else:
        alg.accepted += cnt.accepted

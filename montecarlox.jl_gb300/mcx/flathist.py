"""Multicanonical and Wang-Landau sampling of device lattices (flat-histogram path).

Reference (paths inside MonteCarloX.jl):
  Multicanonical(rng, bins; init)        src/algorithms/multicanonical.jl:9-33
  WangLandau(rng, bins; init, logf)      src/algorithms/wang_landau.jl:9-37
  MulticanonicalEnsemble / update!       src/ensembles/multicanonical.jl:1-43
  WangLandauEnsemble / update!(power)    src/ensembles/wang_landau.jl:1-23
  merge_histograms! / distribute_logweight!  src/algorithms/parallel_multicanonical.jl:38-73
The Wang-Landau stage loop with the flatness test (flatness 0.8, ln f halved to a
final value) is restated from Wang & Landau, PRL 86, 2050 (2001); the reference
ships only the mechanics.
"""
import ctypes as C

import numpy as np

from . import _lib as L
from . import _check, default_context, Philox, ArgumentError, BoundsError

__all__ = ["Bins", "MulticanonicalEnsemble", "WangLandauEnsemble", "Multicanonical", "WangLandau",
           "update_", "sweep_walkers_", "merge_histograms_", "distribute_logweight_", "wang_landau_",
           "flatness"]


class Bins:
    """Integer DiscreteBinning: centers start, start+step, ..., start+step*(nbins-1)."""

    def __init__(self, start, step, nbins):
        self.start, self.step, self.nbins = int(start), int(step), int(nbins)
        if self.step <= 0 or self.nbins <= 0:
            raise ArgumentError("need step > 0 and nbins > 0")

    @classmethod
    def of(cls, bins):
        if isinstance(bins, Bins):
            return bins
        if isinstance(bins, range):
            return cls(bins.start, bins.step, len(bins))
        start, step, n = bins
        return cls(start, step, n)

    def centers(self):
        return self.start + self.step * np.arange(self.nbins, dtype=np.int64)

    def index(self, E):
        """0-based bin of E, or None outside (Julia div semantics)."""
        x = int(E) - self.start
        q = int(x / self.step) if x < 0 else x // self.step
        return q if 0 <= q < self.nbins else None


class _FlatEnsemble:
    def __init__(self, bins, init=0.0, ctx=None):
        self.ctx = ctx or default_context()
        self.bins = Bins.of(bins)
        h = C.c_void_p()
        _check(L.load().mcx_flathist_create(self.ctx.handle, self.bins.start, self.bins.step, self.bins.nbins,
                                            C.byref(h)))
        self.handle = h
        if init != 0.0:
            self.logweight = np.full(self.bins.nbins, float(init))

    @property
    def logweight(self):
        out = np.empty(self.bins.nbins, np.float64)
        _check(L.load().mcx_flathist_get_logweight(self.handle, out.ctypes.data, out.size))
        return out

    @logweight.setter
    def logweight(self, values):
        arr = np.ascontiguousarray(values, np.float64).reshape(-1)
        _check(L.load().mcx_flathist_set_logweight(self.handle, arr.ctypes.data, arr.size))

    @property
    def histogram(self):
        out = np.empty(self.bins.nbins, np.int64)
        _check(L.load().mcx_flathist_get_histogram(self.handle, out.ctypes.data, out.size))
        return out

    @histogram.setter
    def histogram(self, values):
        arr = np.ascontiguousarray(values, np.int64).reshape(-1)
        _check(L.load().mcx_flathist_set_histogram(self.handle, arr.ctypes.data, arr.size))

    def reset_histogram(self):
        _check(L.load().mcx_flathist_reset(self.handle))

    def reweight(self, betas, distribution=False):
        """Canonical averages from the log density of states ln g = -logweight, on the
        device (distribution_from_logdos, src/infrastructure/utils.jl:95-105): returns
        (log Z, <E>, <E^2>) per beta, and with ``distribution`` also the normalised
        distribution over the bins at betas[0]."""
        b = np.ascontiguousarray(np.atleast_1d(betas), np.float64)
        lz, e1, e2 = (np.empty(b.size, np.float64) for _ in range(3))
        dist = np.empty(self.bins.nbins, np.float64) if distribution else None
        _check(L.load().mcx_flathist_reweight(self.handle, b.ctypes.data, b.size, lz.ctypes.data, e1.ctypes.data,
                                              e2.ctypes.data, dist.ctypes.data if distribution else None,
                                              self.bins.nbins if distribution else 0))
        return (lz, e1, e2, dist) if distribution else (lz, e1, e2)

    def close(self):
        if getattr(self, "handle", None):
            L.load().mcx_flathist_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MulticanonicalEnsemble(_FlatEnsemble):
    MODE = L.MUCA
    record_visits = True


class WangLandauEnsemble(_FlatEnsemble):
    MODE = L.WANG_LANDAU

    def __init__(self, bins, init=0.0, logf=1.0, ctx=None):
        super().__init__(bins, init, ctx)
        self.logf = float(logf)


class _FlatAlg:
    def __init__(self, rng, ensemble):
        self.rng = rng if isinstance(rng, Philox) else Philox(rng)
        self.ensemble = ensemble
        self.steps = 0
        self.accepted = 0

    def _reset_hook(self):
        if isinstance(self.ensemble, MulticanonicalEnsemble):
            self.ensemble.reset_histogram()


def Multicanonical(rng, bins, *, init=0.0, ctx=None):
    """Multicanonical(rng, bins; init) -- importance sampling with MUCA weights."""
    ens = bins if isinstance(bins, MulticanonicalEnsemble) else MulticanonicalEnsemble(bins, init, ctx)
    return _FlatAlg(rng, ens)


def WangLandau(rng, bins, *, init=0.0, logf=1.0, ctx=None):
    """WangLandau(rng, bins; init, logf) -- importance sampling with WL adaptation."""
    ens = bins if isinstance(bins, WangLandauEnsemble) else WangLandauEnsemble(bins, init, logf, ctx)
    return _FlatAlg(rng, ens)


def update_(ens, mode="simple", power=0.5):
    """update!(ens): MUCA ln w -= log H (mode :simple); Wang-Landau logf *= power."""
    if isinstance(ens, _FlatAlg):
        ens = ens.ensemble
    if isinstance(ens, MulticanonicalEnsemble):
        if str(mode).lstrip(":") != "simple":
            raise ArgumentError("unsupported mode=%s, currently only :simple" % mode)
        _check(L.load().mcx_flathist_update_muca(ens.handle))
    elif isinstance(ens, WangLandauEnsemble):
        ens.logf *= power
    else:
        raise ArgumentError("update! not implemented for %s" % type(ens).__name__)


def sweep_walkers_(systems, algs, nsweeps):
    """`nsweeps` checkerboard sweeps of every walker.

    systems: list of device lattices.  algs: one algorithm shared by all walkers
    (Multicanonical only; walker i draws from stream rng.stream + i) or one per
    walker."""
    if not isinstance(systems, (list, tuple)):
        systems = [systems]
    shared = not isinstance(algs, (list, tuple))
    alg_list = [algs] if shared else list(algs)
    if not shared and len(alg_list) != len(systems):
        raise ArgumentError("one algorithm per walker, or one shared")
    ens0 = alg_list[0].ensemble
    mode = ens0.MODE
    nw = len(systems)
    lats = (C.c_void_p * nw)(*[s.handle.value for s in systems])
    fhs = (C.c_void_p * len(alg_list))(*[a.ensemble.handle.value for a in alg_list])
    rngs = (L.mcx_rng * nw)()
    for i in range(nw):
        a = alg_list[0] if shared else alg_list[i]
        rngs[i] = L.mcx_rng(a.rng.seed, a.rng.counter, (a.rng.stream + (i if shared else 0)) & 0xFFFFFFFF, 0)
    cnt = (L.mcx_counters * nw)()
    logf = getattr(ens0, "logf", 0.0)
    st = L.load().mcx_flathist_sweep(lats, nw, fhs, len(alg_list), mode, float(logf), rngs, int(nsweeps), cnt)
    if shared:
        alg_list[0].rng.counter += int(nsweeps)
        alg_list[0].steps += sum(c.attempts for c in cnt)
        alg_list[0].accepted += sum(c.accepted for c in cnt)
    else:
        for i, a in enumerate(alg_list):
            a.rng.counter += int(nsweeps)
            a.steps += cnt[i].attempts
            a.accepted += cnt[i].accepted
    _check(st)


def merge_histograms_(dst, srcs):
    arr = (C.c_void_p * len(srcs))(*[s.handle.value for s in srcs])
    _check(L.load().mcx_flathist_merge(dst.handle, arr, len(srcs)))


def distribute_logweight_(src, dsts):
    for d in dsts:
        if d is not src:
            _check(L.load().mcx_flathist_copy_logweight(d.handle, src.handle))


def flatness(ens, threshold=0.8):
    flat = C.c_int()
    ratio = C.c_double()
    _check(L.load().mcx_flathist_flatness(ens.handle, float(threshold), C.byref(flat), C.byref(ratio)))
    return bool(flat.value), ratio.value


def wang_landau_(systems, algs, *, logf_final=1e-8, flat=0.8, check_sweeps=100, max_sweeps_per_stage=None,
                 power=0.5, callback=None):
    """Wang-Landau stages: H := 0, sweep until every walker's histogram is flat
    (min H >= flat * mean H over visited bins), then logf *= power; stop after the
    stage run at logf <= logf_final.  Returns the number of stages run."""
    if not isinstance(algs, (list, tuple)):
        algs = [algs]
    stages = 0
    while True:
        for a in algs:
            a.ensemble.reset_histogram()
        done = 0
        while True:
            sweep_walkers_(systems, algs if len(algs) > 1 else algs[0], check_sweeps)
            done += check_sweeps
            if all(flatness(a.ensemble, flat)[0] for a in algs):
                break
            if max_sweeps_per_stage is not None and done >= max_sweeps_per_stage:
                break
        stages += 1
        if callback is not None:
            callback(stages, algs[0].ensemble.logf, done)
        if algs[0].ensemble.logf <= logf_final:
            return stages
        for a in algs:
            update_(a.ensemble, power=power)

"""Autocorrelation analysis of per-sweep series on the device.

Reference (paths inside MonteCarloX.jl):
  integrated_autocorrelation_time / tau_int    src/measurements/autocorrelations.jl:28-67, :104-110
  integrated_autocorrelation_times             autocorrelations.jl:69-102
  optimize_exchange_interval!                  src/algorithms/parallel_tempering.jl:83-135

The estimator runs on the device (libmcx_cuda, mcx_tau_int and the per-object forms that
read a lattice's, graph's or ladder's series where it already lies); the argument checks
and the retuning of the sweep counts are host logic, as in the reference.
"""
import ctypes as C
import math

import numpy as np

from . import _lib as L
from . import ArgumentError, _check, default_context

__all__ = ["integrated_autocorrelation_time", "integrated_autocorrelation_times", "tau_int", "tau_int_of",
           "optimize_exchange_interval_"]

_QUANTITY = {"energy": 0, "magnetization": 1}


def _batch(traces, min_points, max_lag, c, ctx):
    arrs = [np.ascontiguousarray(t, np.float64).reshape(-1) for t in traces]
    offsets = np.zeros(len(arrs) + 1, np.int64)
    for k, a in enumerate(arrs):
        offsets[k + 1] = offsets[k] + a.size
    values = np.concatenate(arrs) if arrs else np.zeros(1)
    taus = np.zeros(len(arrs), np.float64)
    _check(L.load().mcx_tau_int((ctx or default_context()).handle, values.ctypes.data, offsets.ctypes.data,
                                len(arrs), int(min_points), 0 if max_lag is None else int(max_lag), float(c),
                                taus.ctypes.data))
    return taus


def integrated_autocorrelation_time(samples, *, max_lag=None, c=5.0, ctx=None):
    """tau_int = 1/2 + sum_{t>=1} C(t), truncated at the first C(t) <= 0 or when
    t > c * tau (autocorrelations.jl:28-67); 0.5 for zero variance."""
    x = np.asarray(samples, np.float64).reshape(-1)
    n = x.size
    if n < 2:
        raise ArgumentError("integrated_autocorrelation_time requires at least 2 samples")
    if not c > 0:
        raise ArgumentError("c must be positive")
    cap = n // 2
    if max_lag is not None and not 1 <= int(max_lag) <= cap:
        raise ArgumentError("max_lag must satisfy 1 <= max_lag <= floor(length(samples)/2)")
    return float(_batch([x], 2, max_lag, c, ctx)[0])


tau_int = integrated_autocorrelation_time


def integrated_autocorrelation_times(traces, *, min_points=2, max_lag=None, c=5.0, ctx=None):
    """One tau per trace; NaN for traces with fewer than min_points samples or no lag
    window (autocorrelations.jl:69-102)."""
    if min_points < 2:
        raise ArgumentError("min_points must be >= 2")
    if not c > 0:
        raise ArgumentError("c must be positive")
    if max_lag is not None and int(max_lag) < 1:
        return np.full(len(traces), np.nan)
    return _batch(traces, min_points, max_lag, c, ctx)


def tau_int_of(sys, quantity="energy", *, max_lag=None, c=5.0):
    """tau_int of the energy or magnetization series recorded by the last sweep call of a
    device lattice or graph, computed where the series lies."""
    from .graph import IsingGraphDevice
    out = C.c_double()
    fn = L.load().mcx_graph_tau_int if isinstance(sys, IsingGraphDevice) else L.load().mcx_lattice_tau_int
    _check(fn(sys.handle, _QUANTITY[quantity], 0 if max_lag is None else int(max_lag), float(c), C.byref(out)))
    return out.value


def _retune_exchange_sweeps(sweeps, taus, base_sweeps, min_sweeps, max_sweeps):
    """parallel_tempering.jl:126-140: scale base_sweeps by tau / median(finite taus)."""
    finite = [t for t in taus if math.isfinite(t)]
    tau_ref = float(np.median(finite)) if finite else 1.0
    for i in range(len(sweeps)):
        scale = taus[i] / tau_ref if math.isfinite(taus[i]) else 1.0
        target = int(round(base_sweeps * scale))  # ties to even, as Julia's round
        sweeps[i] = min(max(target, min_sweeps), max_sweeps)
    return sweeps


def optimize_exchange_interval_(pt, local_samples, sweeps_after_exchange, *, base_sweeps, min_sweeps=1,
                                max_sweeps=2 ** 63 - 1, min_points=400, max_lag=200, ctx=None):
    """optimize_exchange_interval!(pt, local_samples, sweeps_after_exchange; ...)
    (parallel_tempering.jl:83-124): tau_int of the energy trace at every ladder position,
    then sweeps_after_exchange[i] = clamp(round(base_sweeps * tau_i / median(tau)), ...).

    ``pt`` is a device ParallelTempering (or the number of positions); ``local_samples``
    are traces grouped per position, or (position, value) tuples (0-based), or None for
    the device series of ``pt``'s last run recorded by position (``pt.record_("position")``).
    Returns the updated ``sweeps_after_exchange`` (one entry per position; the reference
    returns the entry of its own replica)."""
    n = pt if isinstance(pt, int) else pt.npos
    if len(sweeps_after_exchange) != n:
        raise ArgumentError("sweeps_after_exchange must have length size(pt)")
    if local_samples is None:
        taus = pt.tau_int("energy", min_points=min_points, max_lag=max_lag, by="position")
    else:
        if len(local_samples) and isinstance(local_samples[0], tuple):
            grouped = [[] for _ in range(n)]
            for idx, e in local_samples:
                if not 0 <= idx < n:
                    raise ArgumentError("sample index %d out of bounds for %d ladders" % (idx, n))
                grouped[idx].append(float(e))
        else:
            grouped = local_samples
        taus = integrated_autocorrelation_times(grouped, min_points=min_points, max_lag=max_lag, ctx=ctx)
    return _retune_exchange_sweeps(sweeps_after_exchange, list(taus), base_sweeps, min_sweeps, max_sweeps)

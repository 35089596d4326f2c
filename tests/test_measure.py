"""Autocorrelation analysis: the oracle against the reference's own test expectations,
and the host logic of the mirror (CPU)."""
import math

import numpy as np
import pytest

import oracle as O


def _ar1(phi, n, seed):
    rng = np.random.default_rng(seed)
    x = np.empty(n)
    x[0] = rng.normal()
    e = rng.normal(size=n) * math.sqrt(1 - phi * phi)
    for t in range(1, n):
        x[t] = phi * x[t - 1] + e[t]
    return x


def test_oracle_tau_int_reference_expectations():
    # test/test_measurements.jl:151-188 restated with numpy's generator
    assert O.tau_int(np.ones(64)) == 0.5
    white = np.random.default_rng(123).normal(size=4000)
    assert 0.5 <= O.tau_int(white) <= 2.0
    ar = _ar1(0.8, 6000, 123)
    assert 2.5 <= O.tau_int(ar) <= 7.0
    capped = O.tau_int(ar, max_lag=50)
    assert math.isfinite(capped) and capped >= 0.5
    with pytest.raises(ValueError):
        O.tau_int(np.random.default_rng(1).normal(size=20), max_lag=11)
    with pytest.raises(ValueError):
        O.tau_int([1.0])


def test_oracle_tau_int_against_a_direct_formula():
    x = _ar1(0.6, 500, 4)
    c = x - x.mean()
    c0 = (c * c).sum() / len(c)
    tau = 0.5
    for lag in range(1, len(c) // 2 + 1):
        C = ((c[:-lag] * c[lag:]).sum() / (len(c) - lag)) / c0
        if C <= 0 or lag > 5.0 * (tau + C):
            break
        tau += C
    assert abs(O.tau_int(x) - tau) < 1e-12


def test_mirror_argument_checks_and_retune(mcxlib):
    from mcx import measure as Mx
    with pytest.raises(mcxlib.ArgumentError):
        Mx.integrated_autocorrelation_time([1.0])
    with pytest.raises(mcxlib.ArgumentError):
        Mx.integrated_autocorrelation_time(np.zeros(20), max_lag=11)
    with pytest.raises(mcxlib.ArgumentError):
        Mx.integrated_autocorrelation_time(np.zeros(20), c=0.0)
    with pytest.raises(mcxlib.ArgumentError):
        Mx.integrated_autocorrelation_times([np.zeros(20)], min_points=1)
    # a window below 1 gives NaN without a device call (autocorrelations.jl:93-99)
    assert np.isnan(Mx.integrated_autocorrelation_times([np.zeros(20)], max_lag=0)[0])
    # _retune_exchange_sweeps!, src/algorithms/parallel_tempering.jl:126-140
    s = Mx._retune_exchange_sweeps([0, 0, 0], [1.0, 4.0, float("nan")], 10, 2, 50)
    assert s == [4, 16, 10]
    # median of two is their mean: 50.5 -> scales 0.0198, 1.98 -> 0.198 -> clamped to 2, 19.8 -> 20
    s = Mx._retune_exchange_sweeps([0, 0], [1.0, 100.0], 10, 2, 50)
    assert s == [2, 20]
    assert Mx._retune_exchange_sweeps([0], [float("nan")], 7, 1, 9) == [7]
    with pytest.raises(mcxlib.ArgumentError):
        Mx.optimize_exchange_interval_(3, [], [10, 10], base_sweeps=10)

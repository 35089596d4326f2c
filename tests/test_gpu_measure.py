"""Integrated autocorrelation times on the device against the oracle (GPU), for host
traces and for the series the lattices, graphs and ladders keep on the device.  The
device sums in a fixed order of its own; tau agrees with the sequential FP64 oracle to
1e-9 relative (the truncation lags agree on these seeded traces)."""
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _ar1(phi, n, seed):
    rng = np.random.default_rng(seed)
    x = np.empty(n)
    x[0] = rng.normal()
    e = rng.normal(size=n) * math.sqrt(1 - phi * phi)
    for t in range(1, n):
        x[t] = phi * x[t - 1] + e[t]
    return x


def _close(a, b):
    return (math.isnan(a) and math.isnan(b)) or abs(a - b) <= TOL * max(1.0, abs(b))


def test_batch_matches_oracle(gpu):
    from mcx import measure as Mx
    traces = [np.ones(64), np.random.default_rng(1).normal(size=4000), _ar1(0.5, 3000, 2), _ar1(0.8, 6000, 3),
              _ar1(0.95, 20000, 4), _ar1(0.9, 777, 5), np.arange(100.0), np.random.default_rng(6).normal(size=3),
              _ar1(0.99, 50000, 7)]
    taus = Mx.integrated_autocorrelation_times(traces)
    for x, t in zip(traces, taus):
        assert _close(t, O.tau_int(x)), (len(x), t, O.tau_int(x))
    capped = Mx.integrated_autocorrelation_times(traces, max_lag=50, min_points=10)
    for x, t in zip(traces, capped):
        ref = float("nan") if len(x) < 10 else O.tau_int(x, max_lag=min(50, len(x) // 2))
        assert _close(t, ref)
    # test/test_measurements.jl:151-188 on the device
    assert Mx.integrated_autocorrelation_time(np.ones(64)) == 0.5 and Mx.tau_int(np.ones(64)) == 0.5
    assert 0.5 <= Mx.tau_int(traces[1]) <= 2.0
    assert 2.5 <= Mx.tau_int(traces[3]) <= 7.0
    assert Mx.tau_int(traces[3], max_lag=50) >= 0.5
    assert np.isnan(Mx.integrated_autocorrelation_times([np.random.default_rng(8).normal(size=20)], min_points=2,
                                                        max_lag=0)[0])


def test_lattice_and_graph_series_in_place(gpu):
    from mcx import measure as Mx
    sys_ = gpu.BlumeCapel([32, 32], D=0.5, h=0.1)
    gpu.init_(sys_, "random", rng=gpu.Philox(2))
    alg = gpu.Metropolis(gpu.Philox(2), beta=0.5)
    obs = gpu.sweep_(sys_, alg, 3000, record=True).astype(np.float64)
    E = (-(1.0 * obs[:, 0])) - 0.1 * obs[:, 1] + 0.5 * obs[:, 2]
    assert _close(Mx.tau_int_of(sys_, "energy"), O.tau_int(E))
    assert _close(Mx.tau_int_of(sys_, "magnetization", max_lag=100), O.tau_int(obs[:, 1], max_lag=100))
    gpu.sweep_(sys_, alg, 1)
    with pytest.raises(gpu.ArgumentError):
        Mx.tau_int_of(sys_)  # one recorded sweep
    from mcx.graph import IsingGraphDevice
    from graph_cases import from_edges, random_edges
    es = random_edges(800, 2000, 3)
    rp, col, val = from_edges(800, es, np.random.default_rng(4).normal(size=len(es)))
    g = IsingGraphDevice(rp, col, val)
    gpu.init_(g, "random", rng=gpu.Philox(5))
    Es, Ms = gpu.sweep_(g, gpu.Metropolis(gpu.Philox(5), beta=1.5), 2500, record=True)
    assert _close(Mx.tau_int_of(g, "energy"), O.tau_int(Es))
    assert _close(Mx.tau_int_of(g, "magnetization"), O.tau_int(Ms.astype(np.float64)))


def test_ladder_series_by_position_and_exchange_interval(gpu):
    from mcx import measure as Mx
    from mcx.pt import ParallelTempering
    lad = [(8, [0.30, 0.26, 0.22, 0.18]), (16, [0.25, 0.22, 0.19])]
    out = {}
    for mode in ("replica", "position"):
        pt = ParallelTempering(lad, dim=3, seed=9)
        pt.init_(9)
        pt.record_(mode)
        out[mode] = (pt.sweep_(1500, record=True), pt)
    ser_r, _ = out["replica"]
    ser_p, pt = out["position"]
    # the same trajectory: per sweep and ladder the same values, permuted
    for lo, hi in ((0, 4), (4, 7)):
        assert np.array_equal(np.sort(ser_r[:, lo:hi, 0], axis=1), np.sort(ser_p[:, lo:hi, 0], axis=1))
    taus = pt.tau_int("energy", by="position")
    for k in range(pt.nrep):
        assert _close(taus[k], O.tau_int(-ser_p[:, k, 0].astype(np.float64)))
    with pytest.raises(gpu.ArgumentError):
        out["replica"][1].tau_int(by="position")
    sweeps = [10] * pt.npos
    res = Mx.optimize_exchange_interval_(pt, None, sweeps, base_sweeps=10, min_sweeps=2, max_sweeps=50,
                                         min_points=100, max_lag=200)
    assert res is sweeps and all(2 <= v <= 50 for v in sweeps)
    ref_taus = Mx.integrated_autocorrelation_times([-ser_p[:, k, 0].astype(np.float64) for k in range(pt.nrep)],
                                                   min_points=100, max_lag=200)
    assert sweeps == Mx._retune_exchange_sweeps([10] * pt.npos, list(ref_taus), 10, 2, 50)


def test_exchange_interval_reference_case(gpu):
    # test/test_parallel_ensembles.jl:208-228 (positions 0-based here)
    from mcx import measure as Mx
    samples = [(0, 0.0), (0, 0.2), (0, -0.1), (0, 0.1), (0, -0.2),
               (1, 0.0), (1, 2.0), (1, -2.0), (1, 2.0), (1, -2.0)]
    sweeps = [10, 10]
    Mx.optimize_exchange_interval_(2, samples, sweeps, base_sweeps=10, min_sweeps=2, max_sweeps=50, min_points=2,
                                   max_lag=2)
    assert all(2 <= v <= 50 for v in sweeps) and sweeps[1] >= sweeps[0]


# ---- reweighting from a log density of states on the device (utils.jl:54-105) ----

def _reweight_ref(lng, centers, beta):
    """FP64 numpy: log Z, <E>, <E^2> and the distribution over the finite bins, from
    weights shifted by their maximum and pairwise sums (a sequential logaddexp over
    millions of bins drifts by ~1e-8 and would scale every probability by that)."""
    w = lng - beta * centers
    m = np.isfinite(w)
    wmax = w[m].max()
    q = np.zeros_like(w)
    q[m] = np.exp(w[m] - wmax)
    z = q.sum()
    p = q / z
    return wmax + np.log(z), float((q * centers).sum() / z), float((q * centers * centers).sum() / z), p


def test_reweight_exact_ising_8x8(gpu):
    """The exact 8x8 Ising density of states (Beale 1996, the reference's ising2d_exact
    data) reweighted on the device: log Z, <E>, <E^2> and the distribution at several
    betas against FP64 numpy, and the distribution against distribution_from_logdos."""
    import json
    import os
    from mcx import analysis as A
    from mcx import flathist as F
    d = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ising2d_8x8_logdos.json")))
    ens = F.MulticanonicalEnsemble((-128, 4, 65))
    lng = np.full(65, -np.inf)
    for E, g in d["energy_logdos"]:
        lng[(E + 128) // 4] = g
    ens.logweight = -lng  # ln g = -logweight; impossible energies are +inf weights
    centers = ens.bins.centers().astype(np.float64)
    betas = [0.1, 0.3, 0.4406868, 0.6, 1.0]
    lz, e1, e2, dist = ens.reweight(betas, distribution=True)
    for k, b in enumerate(betas):
        rlz, re1, re2, rp = _reweight_ref(lng, centers, b)
        assert abs(lz[k] - rlz) <= 1e-12 * abs(rlz) + 1e-12
        assert abs(e1[k] - re1) <= 1e-11 * abs(re1)
        assert abs(e2[k] - re2) <= 1e-11 * abs(re2)
        if k == 0:
            np.testing.assert_allclose(dist, rp, rtol=1e-11, atol=1e-300)
            np.testing.assert_allclose(dist, A.distribution_from_logdos(centers, lng, b), rtol=1e-11, atol=1e-300)
    assert abs(np.log(np.exp(lng[np.isfinite(lng)]).sum()) - np.log(2.0) * 64) < 1e-9  # sum g = 2^64


@pytest.mark.parametrize("nbins,step,nbeta", [(4 * 1024 * 1024 + 1, 1, 3), (100003, 4, 300)])
def test_reweight_many_bins(gpu, nbins, step, nbeta):
    """A smooth log density of states over millions of bins (the Blume-Capel L=1024 range)
    and a scan of many betas: every block and both grid dimensions in use."""
    from mcx import flathist as F
    start = -nbins // 2 * step
    ens = F.MulticanonicalEnsemble((start, step, nbins))
    x = np.linspace(-1.0, 1.0, nbins)
    lng = nbins * 0.5 * (1.0 - x * x) + np.sin(37.0 * x)
    lng[::97] = -np.inf  # some impossible energies
    ens.logweight = -lng
    centers = ens.bins.centers().astype(np.float64)
    betas = np.linspace(-0.5, 0.5, nbeta)
    lz, e1, e2 = ens.reweight(betas)
    for k in range(0, nbeta, max(1, nbeta // 7)):
        rlz, re1, re2, _ = _reweight_ref(lng, centers, betas[k])
        assert abs(lz[k] - rlz) <= 1e-12 * abs(rlz), k
        assert abs(e1[k] - re1) <= 1e-10 * np.sqrt(re2), k  # sums of E p cancel: scale by rms E
        assert abs(e2[k] - re2) <= 1e-9 * abs(re2), k


def test_reweight_errors(gpu):
    from mcx import flathist as F
    ens = F.MulticanonicalEnsemble((0, 1, 8))
    ens.logweight = np.full(8, np.inf)  # no finite bin
    with pytest.raises(gpu.ArgumentError):
        ens.reweight([0.5])
    ens.logweight = np.zeros(8)
    with pytest.raises(gpu.ArgumentError):
        ens.reweight([np.nan])
    lz, e1, e2 = ens.reweight([0.0])
    assert abs(lz[0] - np.log(8.0)) < 1e-14 and abs(e1[0] - 3.5) < 1e-14

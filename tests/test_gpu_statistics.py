"""Statistical level of correctness (GPU): device checkerboard sweeps against the
reference's default sequential random-site sweep (oracle mode ii) for E, |M| and the
Binder cumulant within 3 sigma of binned error bars, and 2-D Ising against Onsager."""
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _seq_series(L, beta, seed, nsweeps, therm):
    N = int(np.prod(L))
    s = O.init_random(O.ISING, L, seed)
    a = 0
    O.seq_attempts(s, O.ISING, L, O.METROPOLIS, beta, seed, attempt0=a, nattempts=N * therm)
    a += N * therm
    P = np.empty(nsweeps)
    M = np.empty(nsweeps)
    for k in range(nsweeps):
        O.seq_attempts(s, O.ISING, L, O.METROPOLIS, beta, seed, attempt0=a, nattempts=N)
        a += N
        p, m, _ = O.observables(s, L)
        P[k], M[k] = p, m
    return -P / N, M / N


def _dev_series(mcx, L, beta, seed, nsweeps, therm, alg="metropolis", start="random"):
    N = int(np.prod(L))
    sys_ = mcx.Ising(L)
    if start == "random":
        mcx.init_(sys_, "random", rng=mcx.Philox(seed))
    else:
        mcx.init_(sys_, start)
    a = {"metropolis": mcx.Metropolis, "glauber": mcx.Glauber, "heatbath": mcx.HeatBath}[alg](mcx.Philox(seed + 1),
                                                                                            beta=beta)
    mcx.sweep_(sys_, a, therm)
    obs = mcx.sweep_(sys_, a, nsweeps, record=True)
    return -obs[:, 0] / N, obs[:, 1] / N


def _compare(x, y, what):
    from mcx.analysis import binning_error
    ex, ey = binning_error(x), binning_error(y)
    d = abs(x.mean() - y.mean())
    assert d < 3 * math.hypot(ex, ey) + 1e-12, (what, x.mean(), y.mean(), ex, ey)


@pytest.mark.parametrize("beta", [0.35, 0.4407, 0.5])
def test_device_matches_sequential_reference_order(gpu, beta):
    from mcx.analysis import binder_cumulant
    L = [16, 16]
    e_s, m_s = _seq_series(L, beta, 101, 40000, 2000)
    e_d, m_d = _dev_series(gpu, L, beta, 202, 40000, 2000)
    _compare(e_s, e_d, "E")
    _compare(np.abs(m_s), np.abs(m_d), "|M|")
    u_s, eu_s = binder_cumulant(m_s)
    u_d, eu_d = binder_cumulant(m_d)
    assert abs(u_s - u_d) < 3 * math.hypot(eu_s, eu_d) + 1e-12, (u_s, u_d, eu_s, eu_d)


@pytest.mark.parametrize("beta,alg", [(0.3, "metropolis"), (0.6, "metropolis"), (0.3, "glauber"), (0.6, "heatbath")])
def test_onsager(gpu, beta, alg):
    """L=256 away from beta_c: finite-size corrections are far below the error bars.
    The ordered phase starts ordered: from a random start the domains of a 256^2
    lattice need far more sweeps to coarsen than the run has."""
    from mcx.analysis import BETA_C, binning_error, onsager_energy_per_site, onsager_magnetization
    e, m = _dev_series(gpu, [256, 256], beta, 7, 4000, 1000, alg, start="up" if beta > BETA_C else "random")
    u = onsager_energy_per_site(beta)
    err = binning_error(e)
    assert abs(e.mean() - u) < 3 * err + 2e-4, (e.mean(), u, err)
    if beta > 0.5:
        mm = onsager_magnetization(beta)
        em = binning_error(np.abs(m))
        assert abs(np.abs(m).mean() - mm) < 3 * em + 2e-4, (np.abs(m).mean(), mm, em)


def test_exact_dos_distribution_l8(gpu):
    """Device energy histogram at L=8 against distribution_exact_ising2D(8, beta)
    (SpinSystems/src/ising2d_exact.jl:35-40) -- chi-square over the populated bins."""
    import json
    import os
    d = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ising2d_8x8_logdos.json")))
    E = np.array([e for e, _ in d["energy_logdos"]], float)
    beta = 0.4
    lw = np.array([v for _, v in d["energy_logdos"]]) - beta * E
    p = np.exp(lw - lw.max())
    p /= p.sum()
    e, _ = _dev_series(gpu, [8, 8], beta, 3, 200000, 1000)
    Es = np.rint(e * 64).astype(int)
    # thin by 10 sweeps to reduce correlation, then chi-square on bins with >= 20 expected counts
    Es = Es[::10]
    n = len(Es)
    counts = np.array([(Es == x).sum() for x in E.astype(int)])
    mask = p * n >= 20
    chi2 = (((counts - n * p) ** 2) / (n * p))[mask].sum()
    dof = mask.sum() - 1
    assert chi2 < dof + 5 * math.sqrt(2 * dof), (chi2, dof)


def test_kaufman_configured_l64_chain(gpu):
    """The configured small run: L=64, Philox key 42, Metropolis at beta 0.4407 (next to
    beta_c), 10^3 thermalisation sweeps then 10^4 recorded: the mean energy per site within
    3 sigma (binning) of the exact finite-torus value (Kaufman 1949)."""
    from mcx.analysis import binning_error, kaufman_ising2d
    L, beta = 64, 0.4407
    sys_ = gpu.Ising([L, L])
    gpu.init_(sys_, "random", rng=gpu.Philox(42))
    a = gpu.Metropolis(gpu.Philox(42), beta=beta)
    gpu.sweep_(sys_, a, 1000)
    obs = gpu.sweep_(sys_, a, 10000, record=True)
    e = -obs[:, 0] / (L * L)
    exact = kaufman_ising2d(L, L, beta)[1] / (L * L)
    err = binning_error(e, min_bins=16)
    assert abs(e.mean() - exact) < 3 * err, (e.mean(), exact, err)


@pytest.mark.parametrize("L", [32, 64])
def test_kaufman_independent_chains(gpu, L):
    """64 independent chains (one batched call, streams 0..63) of the same workload: the
    mean energy per site over the chains within 3 standard errors of the chain means of
    Kaufman's exact value at beta 0.4407."""
    from mcx.analysis import kaufman_ising2d
    beta, nch = 0.4407, 64
    chains = [gpu.Ising([L, L]) for _ in range(nch)]
    for i, c in enumerate(chains):
        gpu.init_(c, "random", rng=gpu.Philox(42, i))
    algs = [gpu.Metropolis(gpu.Philox(42, i), beta=beta) for i in range(nch)]
    gpu.sweep_batch_(chains, algs, 1000)
    obs = gpu.sweep_batch_(chains, algs, 10000, record=True)
    means = np.array([(-o[:, 0] / (L * L)).mean() for o in obs])
    exact = kaufman_ising2d(L, L, beta)[1] / (L * L)
    se = means.std(ddof=1) / math.sqrt(nch)
    assert abs(means.mean() - exact) < 3 * se, (means.mean(), exact, se)
    for c in chains:
        c.close()

"""The configured workloads at their configured sizes, against the oracle bit for bit (GPU).

* 2-D Ising L=4096 (seed 7): Metropolis and Glauber at beta 0.30 / 0.4407 / 0.60, and the
  heat bath at the same betas, on the int8 and the 64-spins-per-word layouts.
* 2-D Blume-Capel L=1024, J=1, D=1, 4,194,305 bins of width 1 (E in [-N, 3N]): walkers on
  one shared Multicanonical table, walkers with their own Wang-Landau tables, and one full
  wave of 608 walkers on one shared table (the flat-histogram bench shape).
* Batched parallel tempering: 256 3-D replicas in five ladders of sides 16/24/32/48/64
  (52, 51, 51, 51, 51 replicas), geometric betas 0.20 -> 0.25 per ladder, an exchange after
  every sweep, in the persistent and in the plain form.
"""
import hashlib
import multiprocessing as mp
import os

import numpy as np
import pytest

import oracle as O
from oracle_runs import ALG, muca_walker_range, oracle_pt

pytestmark = pytest.mark.gpu

# ------------------------------------------------------------------ 2-D L=4096 --
L2 = [4096, 4096]
SEED2 = 7
_init_cache = {}


def _init4096():
    if "s" not in _init_cache:
        _init_cache["s"] = O.init_random(O.ISING, L2, SEED2)
    return _init_cache["s"]


C2_CASES = [(a, b) for a in ("metropolis", "glauber", "heatbath") for b in (0.30, 0.4407, 0.60)]


@pytest.mark.parametrize("alg,beta", C2_CASES)
def test_ising_L4096_two_sweeps(gpu, alg, beta):
    s = _init4096().copy()
    oobs, att, acc = O.cb_sweep(s, O.ISING, L2, ALG[alg], beta, SEED2, nsweeps=2)
    for layout in ("int8", "msc64"):
        sys_ = gpu.Ising(L2, layout=layout)
        gpu.init_(sys_, "random", rng=gpu.Philox(SEED2))
        a = {"metropolis": gpu.Metropolis, "glauber": gpu.Glauber, "heatbath": gpu.HeatBath}[alg](
            gpu.Philox(SEED2), beta=beta)
        obs = gpu.sweep_(sys_, a, 2, record=True)
        assert np.array_equal(obs, oobs), layout
        assert a.steps == att
        assert (a.flips if alg == "heatbath" else a.accepted) == acc, layout
        assert np.array_equal(sys_.spins, s), layout
        assert gpu.observables(sys_) == gpu.observables(sys_, full=True)
        sys_.close()


# ------------------------------------------------------- Blume-Capel L=1024 --
LBC = [1024, 1024]
NBC = LBC[0] * LBC[1]
BINS = (-NBC, 1, 4 * NBC + 1)
SEED3 = 11


def _lnw_beta(beta=0.35):
    start, step, nb = BINS
    return -beta * (start + step * np.arange(nb)).astype(np.float64)


def _bc_walkers(gpu, n):
    ws = []
    for i in range(n):
        w = gpu.BlumeCapel(LBC, D=1.0)
        gpu.init_(w, "random", rng=gpu.Philox(SEED3, i))
        ws.append(w)
    return ws


def _series(gpu, sys_, n):
    out = np.zeros((n, 3), np.int64)
    gpu._check(gpu._lib.load().mcx_read_series(sys_.handle, out.ctypes.data, n))
    return out


def test_bc_L1024_shared_multicanonical(gpu):
    """Four walkers on one shared 4,194,305-bin table, two sweeps: spins, series, H, ln g."""
    from mcx import flathist as F
    nw, nsw = 4, 2
    lnw0 = _lnw_beta()
    walkers = _bc_walkers(gpu, nw)
    ens = F.MulticanonicalEnsemble(BINS)
    ens.logweight = lnw0
    alg = F.Multicanonical(gpu.Philox(SEED3), ens)
    F.sweep_walkers_(walkers, alg, nsw)
    H, res = muca_walker_range((LBC, 1.0, BINS, lnw0, SEED3, 0, nw, nsw))
    assert np.array_equal(ens.histogram, H)
    assert np.array_equal(ens.logweight, lnw0)
    for i, (rc, st, ac, digest, obs) in enumerate(res):
        assert rc == O.OK
        assert hashlib.sha1(walkers[i].spins.tobytes()).hexdigest() == digest, i
        assert np.array_equal(_series(gpu, walkers[i], nsw), obs), i
    assert (alg.steps, alg.accepted) == (sum(r[1] for r in res), sum(r[2] for r in res))
    for w in walkers:
        w.close()
    ens.close()


def test_bc_L1024_per_walker_wang_landau(gpu):
    """Three walkers with their own 4,194,305-bin Wang-Landau tables (ln f = 1), two sweeps:
    the FP64 ln g of every walker bit for bit."""
    from mcx import flathist as F
    nw, nsw = 3, 2
    walkers = _bc_walkers(gpu, nw)
    algs = [F.WangLandau(gpu.Philox(SEED3, i), F.WangLandauEnsemble(BINS, logf=1.0)) for i in range(nw)]
    F.sweep_walkers_(walkers, algs, nsw)
    start, step, nb = BINS
    for i in range(nw):
        s = O.init_random(O.BC, LBC, SEED3, i)
        lnw = np.zeros(nb)
        H = np.zeros(nb, np.int64)
        rc, obs, st, ac = O.flathist_sweep(s, O.BC, LBC, O.WL, lnw, H, start, step, 1.0, SEED3, stream=i,
                                           nsweeps=nsw, D=1.0)
        assert rc == O.OK
        e = algs[i].ensemble
        assert np.array_equal(e.logweight, lnw), i
        assert np.array_equal(e.histogram, H), i
        assert np.array_equal(walkers[i].spins, s), i
        assert np.array_equal(_series(gpu, walkers[i], nsw), obs), i
        assert (algs[i].steps, algs[i].accepted) == (st, ac)
        walkers[i].close()
        e.close()


def test_bc_L1024_full_wave_shared_table(gpu):
    """One wave of walkers (four per SM: 608 on a GB300) on one shared table, one sweep:
    the merged histogram, the unchanged ln g, the counters and every walker's spins and
    series against the oracle (walkers split over a spawn process pool)."""
    import torch
    from mcx import flathist as F
    nw = 4 * torch.cuda.get_device_properties(0).multi_processor_count
    lnw0 = _lnw_beta()
    walkers = _bc_walkers(gpu, nw)
    ens = F.MulticanonicalEnsemble(BINS)
    ens.logweight = lnw0
    alg = F.Multicanonical(gpu.Philox(SEED3), ens)
    F.sweep_walkers_(walkers, alg, 1)
    Hd = ens.histogram
    assert np.array_equal(ens.logweight, lnw0)
    digests = [hashlib.sha1(w.spins.tobytes()).hexdigest() for w in walkers]
    series = [_series(gpu, w, 1) for w in walkers]
    for w in walkers:
        w.close()
    ens.close()
    nproc = max(1, min(16, os.cpu_count() or 1))
    bounds = np.linspace(0, nw, nproc + 1).astype(int)
    jobs = [(LBC, 1.0, BINS, lnw0, SEED3, int(bounds[k]), int(bounds[k + 1]), 1) for k in range(nproc)]
    with mp.get_context("spawn").Pool(nproc) as pool:
        parts = pool.map(muca_walker_range, jobs)
    H = np.zeros_like(Hd)
    res = []
    for h, r in parts:
        H += h
        res += r
    assert np.array_equal(Hd, H)
    assert all(r[0] == O.OK for r in res)
    assert digests == [r[3] for r in res]
    for i in range(nw):
        assert np.array_equal(series[i], res[i][4]), i
    assert (alg.steps, alg.accepted) == (sum(r[1] for r in res), sum(r[2] for r in res))


# ------------------------------------------------------------- the PT ladder --
PT_SIZES = [16, 24, 32, 48, 64]
PT_COUNTS = [52, 51, 51, 51, 51]
PT_SEED = 7
PT_SWEEPS = 3
_pt_cache = {}


def _pt_ladders():
    from mcx.pt import set_betas
    return [(L, set_betas(n, 0.20, 0.25, ":geometric")) for L, n in zip(PT_SIZES, PT_COUNTS)]


def _pt_oracle():
    if "r" not in _pt_cache:
        _pt_cache["r"] = oracle_pt(_pt_ladders(), 3, "metropolis", PT_SEED, PT_SWEEPS, 1)
    return _pt_cache["r"]


@pytest.mark.parametrize("mode", ["persistent", "plain"])
def test_pt_256_replicas_configured_ladder(gpu, mode):
    from mcx.pt import ParallelTempering
    ladders = _pt_ladders()
    pt = ParallelTempering(ladders, dim=3, seed=PT_SEED)
    assert pt.nrep == 256
    pt.init_(PT_SEED)
    series = pt.sweep_(PT_SWEEPS, alg="metropolis", exchange_every=1, mode=mode, record=True)
    spins, oseries, opos, ostage, osteps, oacc = _pt_oracle()
    assert np.array_equal(series, oseries)
    assert np.array_equal(pt.positions, opos)
    assert pt.stage == ostage
    s, a = pt.counters()
    assert np.array_equal(s, osteps) and np.array_equal(a, oacc)
    for r in range(pt.nrep):
        assert np.array_equal(pt.spins(r), spins[r]), r
    pt.close()


# ------------------------------- FP64 decisions against the reference's literal rule --
def _u53(hi, lo):
    return float((int(hi) << 21) | (int(lo) >> 11)) * 2.0 ** -53


def test_pt_exchange_replay_and_literal_rule(gpu):
    """400 sweeps of the configured ladder with an exchange after every sweep.  The host
    replays every exchange decision from the device's recorded energies and the exchange
    uniforms (Philox(seed, (pair, sweep lo, sweep hi16 | 4<<24, ladder)), words 0-1): the
    device's rule lr > 0 || log(U) < lr reproduces the final positions, stage and edge
    counters, and the reference's literal rule lr > 0 || U < exp(lr)
    (src/algorithms/replica_exchange.jl:110-115) takes the same decision every time."""
    import math
    from mcx.pt import ParallelTempering
    ladders = _pt_ladders()
    nsw = 400
    pt = ParallelTempering(ladders, dim=3, seed=PT_SEED)
    pt.init_(PT_SEED)
    series = pt.sweep_(nsw, alg="metropolis", exchange_every=1, record=True)
    key = np.array([PT_SEED & 0xFFFFFFFF, PT_SEED >> 32], np.uint32)
    first = np.cumsum([0] + [len(b) for _, b in ladders])
    pos = [np.arange(len(b)) for _, b in ladders]
    steps = [np.zeros(len(b) - 1, np.uint64) for _, b in ladders]
    acc = [np.zeros(len(b) - 1, np.uint64) for _, b in ladders]
    stage, ndec, disagree = 0, 0, 0
    for t in range(nsw):
        for l, (_, b) in enumerate(ladders):
            n = len(b)
            rep = np.empty(n, np.int64)
            rep[pos[l]] = np.arange(n)
            for p in range(stage % 2, n - 1, 2):
                ri, rj = rep[p], rep[p + 1]
                w = O.philox([p, t & 0xFFFFFFFF, ((t >> 32) & 0xFFFF) | (4 << 24), l], key)
                U = _u53(w[0], w[1])
                xi = -float(series[t, first[l] + ri, 0])
                xj = -float(series[t, first[l] + rj, 0])
                bi, bj = b[p], b[p + 1]
                lr = (((-bi) * xj) - ((-bi) * xi)) + (((-bj) * xi) - ((-bj) * xj))
                d_dev = (lr > 0) or (O.log(U) < lr)
                d_ref = (lr > 0) or (U < math.exp(lr))
                ndec += 1
                disagree += d_dev != d_ref
                steps[l][p] += 1
                if d_dev:
                    acc[l][p] += 1
                    pos[l][ri], pos[l][rj] = p + 1, p
        stage = 1 - stage
    assert ndec > 50000
    assert disagree == 0
    assert np.array_equal(pt.positions, np.concatenate(pos))
    assert pt.stage == stage
    s, a = pt.counters()
    assert np.array_equal(s, np.concatenate(steps)) and np.array_equal(a, np.concatenate(acc))
    pt.close()


def test_muca_update_configured_bins_against_numpy(gpu):
    """update!(::MulticanonicalEnsemble) over the 4,194,305 bins: bit for bit with the
    oracle, and within 1 ulp of log(H) plus the rounding of the subtraction of numpy's
    lnw - log(H) (src/ensembles/multicanonical.jl:37-41) on every bin."""
    from mcx import flathist as F
    rng = np.random.default_rng(17)
    start, step, nb = BINS
    E = start + step * np.arange(nb, dtype=np.float64)
    lnw = -0.35 * E - 1e-7 * E * E
    H = np.zeros(nb, np.int64)
    band = slice(NBC // 2, 3 * NBC)  # the visited energies of a production run
    H[band] = rng.poisson(rng.uniform(0.5, 2e6, size=H[band].size))
    ens = F.MulticanonicalEnsemble(BINS)
    ens.logweight = lnw
    ens.histogram = H
    F.update_(ens)
    got = ens.logweight
    ens.close()
    orc = lnw.copy()
    O.muca_update(orc, H)
    assert np.array_equal(got, orc)
    m = H > 0
    logh = np.log(H[m].astype(np.float64))
    ref = lnw[m] - logh
    bound = np.spacing(np.abs(logh)) + np.spacing(np.abs(ref))
    assert np.all(np.abs(got[m] - ref) <= bound)
    assert np.array_equal(got[~m], lnw[~m])


# ------------------------------------------- schedules of the persistent ladder kernel --
def test_pt_every_schedule_is_bit_exact(gpu):
    """Every schedule the autotuner may choose (blocks per SM x widest chunk 16 / 8 / 4 x
    warp-split weights) gives the oracle's run of the configured ladder bit for bit."""
    from mcx.pt import ParallelTempering
    ladders = _pt_ladders()
    spins, oseries, opos, ostage, osteps, oacc = _pt_oracle()
    probe = ParallelTempering(ladders, dim=3, seed=PT_SEED)
    bmax = probe.schedule[3]
    probe.close()
    for b in range(1, bmax + 1):
        for v in (16, 8, 4):
            for w in (0, 1, 2):
                pt = ParallelTempering(ladders, dim=3, seed=PT_SEED)
                pt.set_schedule(b, v, w)
                assert pt.schedule[:3] == (b, v, w)
                pt.init_(PT_SEED)
                series = pt.sweep_(PT_SWEEPS, alg="metropolis", exchange_every=1, record=True)
                assert np.array_equal(series, oseries), (b, v, w)
                assert np.array_equal(pt.positions, opos) and pt.stage == ostage, (b, v, w)
                s, a = pt.counters()
                assert np.array_equal(s, osteps) and np.array_equal(a, oacc), (b, v, w)
                assert np.array_equal(pt.spins(255), spins[255]), (b, v, w)
                pt.close()


def test_pt_autotune_keeps_the_run(gpu):
    """Autotuning times the schedules on the ladder's own state and restores it: a ladder
    tuned between two runs ends exactly where an untuned twin ends."""
    from mcx.pt import ParallelTempering
    lad = [(16, [0.25, 0.24, 0.23, 0.22]), (24, [0.23, 0.22, 0.21]), (32, [0.22, 0.21])]
    a = ParallelTempering(lad, dim=3, seed=9)
    b = ParallelTempering(lad, dim=3, seed=9)
    a.init_(9)
    b.init_(9)
    a.sweep_(3, alg="heatbath", exchange_every=2)
    b.sweep_(3, alg="heatbath", exchange_every=2)
    before = (a.positions.copy(), a.stage, a.counters(), a.observables(), [a.spins(r) for r in range(a.nrep)])
    bb, vv, ww, ns = a.autotune_(alg="heatbath", exchange_every=2, sweeps=5)
    assert a.schedule[:3] == (bb, vv, ww) and ns > 0
    after = (a.positions, a.stage, a.counters(), a.observables(), [a.spins(r) for r in range(a.nrep)])
    assert np.array_equal(before[0], after[0]) and before[1] == after[1]
    for x, y in zip(before[2] + before[3], after[2] + after[3]):
        assert np.array_equal(x, y)
    for x, y in zip(before[4], after[4]):
        assert np.array_equal(x, y)
    sa = a.sweep_(4, alg="heatbath", exchange_every=2, record=True)
    sb = b.sweep_(4, alg="heatbath", exchange_every=2, record=True)
    assert np.array_equal(sa, sb) and np.array_equal(a.positions, b.positions)
    for r in range(a.nrep):
        assert np.array_equal(a.spins(r), b.spins(r))
    a.close()
    b.close()

"""Multicanonical / Wang-Landau sweeps on the device against the oracle (GPU)."""
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _walkers(mcx, model, L, n, seed, D=0.0):
    sysl = []
    spins = []
    for i in range(n):
        if model == O.ISING:
            s = mcx.Ising(L)
        else:
            s = mcx.BlumeCapel(L, D=D)
        mcx.init_(s, "random", rng=mcx.Philox(seed, i))
        sysl.append(s)
        spins.append(O.init_random(model, L, seed, i))
    return sysl, spins


CASES = [
    # model, L, D, bins (start, step, nbins), mode, nwalkers, shared, logf, nsweeps, lnw kind
    (O.ISING, [8, 8], 0.0, (-128, 4, 65), "muca", 1, True, 0.0, 30, "beta"),
    (O.ISING, [8, 8], 0.0, (-128, 4, 65), "muca", 5, True, 0.0, 20, "beta"),
    (O.ISING, [8, 8], 0.0, (-128, 4, 65), "wl", 1, False, 1.0, 25, "flat"),
    (O.ISING, [16, 8], 0.0, (-256, 4, 129), "wl", 3, False, 0.25, 10, "flat"),
    (O.ISING, [4, 4, 4], 0.0, (-192, 4, 97), "muca", 2, False, 0.0, 15, "beta"),
    (O.BC, [8, 8], 1.0, (-64, 1, 257), "wl", 2, False, 0.5, 12, "flat"),
    (O.BC, [12, 8], 1.0, (-96, 1, 385), "muca", 3, True, 0.0, 10, "beta"),
    # more bins than the 512-bin shared-memory window: the energy drifts and the window moves
    (O.BC, [32, 32], 1.0, (-1024, 1, 4097), "muca", 4, True, 0.0, 20, "beta"),
    (O.ISING, [32, 32], 0.0, (-2048, 1, 4097), "wl", 2, False, 0.05, 10, "beta"),
    # Wang-Landau with ln f a power of two holds windows of multiples of ln f as integers: with
    # moving windows (Ising and Blume-Capel), and weights that are not such multiples (the
    # FP64 form is kept)
    (O.ISING, [32, 32], 0.0, (-2048, 1, 4097), "wl", 2, False, 2.0 ** -10, 10, "flat"),
    (O.BC, [32, 32], 1.0, (-1024, 1, 4097), "wl", 2, False, 0.5, 15, "flat"),
    (O.BC, [32, 32], 1.0, (-1024, 1, 4097), "wl", 2, False, 1.0, 10, "beta"),
    (O.ISING, [8, 8, 8], 0.0, (-1536, 2, 1537), "muca", 3, True, 0.0, 6, "beta"),
    # bin width not a power of two: the general 64-bit binning path
    (O.ISING, [16, 16], 0.0, (-512, 12, 86), "muca", 2, True, 0.0, 10, "beta"),
]


@pytest.mark.parametrize("model,L,D,bins,mode,nw,shared,logf,nsweeps,lw", CASES)
def test_flathist_parity(gpu, model, L, D, bins, mode, nw, shared, logf, nsweeps, lw):
    from mcx import flathist as F
    start, step, nb = bins
    centers = start + step * np.arange(nb)
    lnw0 = -0.35 * centers.astype(np.float64) if lw == "beta" else np.zeros(nb)
    seed = 77
    sysl, spins = _walkers(gpu, model, L, nw, seed, D)
    if mode == "muca":
        make = lambda: F.MulticanonicalEnsemble(bins)
    else:
        make = lambda: F.WangLandauEnsemble(bins, logf=logf)
    if shared:
        ens = make()
        ens.logweight = lnw0
        alg = F.Multicanonical(gpu.Philox(seed), ens)
        algs = alg
    else:
        algs = []
        for i in range(nw):
            e = make()
            e.logweight = lnw0
            algs.append((F.Multicanonical if mode == "muca" else F.WangLandau)(gpu.Philox(seed, i), e))
    F.sweep_walkers_(sysl, algs, nsweeps)
    # oracle
    omode = O.MUCA if mode == "muca" else O.WL
    if shared:
        olnw = lnw0.copy()
        oH = np.zeros(nb, np.int64)
    tot_st = tot_ac = 0
    for i in range(nw):
        if not shared:
            olnw = lnw0.copy()
            oH = np.zeros(nb, np.int64)
        rc, obs, st, ac = O.flathist_sweep(spins[i], model, L, omode, olnw, oH, start, step, logf, seed, stream=i,
                                           nsweeps=nsweeps, D=D)
        assert rc == O.OK
        assert np.array_equal(sysl[i].spins, spins[i])
        series = np.zeros((nsweeps, 3), np.int64)
        gpu._check(gpu._lib.load().mcx_read_series(sysl[i].handle, series.ctypes.data, nsweeps))
        assert np.array_equal(series, obs)
        if not shared:
            e = algs[i].ensemble
            assert np.array_equal(e.histogram, oH)
            assert np.array_equal(e.logweight, olnw)  # FP64, bit for bit
            assert (algs[i].steps, algs[i].accepted) == (st, ac)
        tot_st += st
        tot_ac += ac
    if shared:
        assert np.array_equal(algs.ensemble.histogram, oH)
        assert np.array_equal(algs.ensemble.logweight, olnw)
        assert (algs.steps, algs.accepted) == (tot_st, tot_ac)


def test_out_of_range_is_bounds_error(gpu):
    from mcx import flathist as F
    L = [8, 8]
    sysl, spins = _walkers(gpu, O.ISING, L, 1, 3)
    up = np.ones(64, np.int8)  # E = -128
    sysl[0].spins = up
    e2 = F.MulticanonicalEnsemble((-128, 4, 3))  # E in {-128, -124, -120}; first flip gives -120, then more
    alg = F.Multicanonical(gpu.Philox(9), e2)
    with pytest.raises(gpu.BoundsError):
        F.sweep_walkers_([sysl[0]], alg, 5)
    s = up.copy()
    lnw = np.zeros(3)
    H = np.zeros(3, np.int64)
    rc, _, st, ac = O.flathist_sweep(s, O.ISING, L, O.MUCA, lnw, H, -128, 4, 0.0, 9, nsweeps=5)
    assert rc == O.ERR_RANGE
    assert np.array_equal(sysl[0].spins, s)
    assert np.array_equal(e2.histogram, H)
    assert (alg.steps, alg.accepted) == (st, ac)
    assert gpu.observables(sysl[0]) == O.observables(s, L)


def test_muca_update_flatness_merge(gpu):
    from mcx import flathist as F
    rng = np.random.default_rng(5)
    H = rng.integers(0, 1000, 4097).astype(np.int64)
    H[::7] = 0
    lnw = rng.normal(size=4097)
    e = F.MulticanonicalEnsemble((0, 1, 4097))
    e.logweight = lnw
    e.histogram = H
    F.update_(e)
    ref = lnw.copy()
    O.muca_update(ref, H)
    assert np.array_equal(e.logweight, ref)  # bit for bit: same log restated on both sides
    vis = (H > 0).astype(np.uint8)
    flat, ratio = F.flatness(e, 0.8)
    oflat, oratio = O.wl_flat(H, vis, 0.8)
    assert flat == oflat and ratio == oratio
    e2 = F.MulticanonicalEnsemble((0, 1, 4097))
    e2.histogram = H
    F.merge_histograms_(e2, [e, e])
    assert np.array_equal(e2.histogram, 3 * H)
    F.distribute_logweight_(e, [e2])
    assert np.array_equal(e2.logweight, ref)


def test_wang_landau_driver_converges_on_small_ising(gpu):
    """WL stages on the 4x4 Ising model recover ln g up to a constant (exact DOS by enumeration)."""
    from mcx import flathist as F
    L = [4, 4]
    # exact density of states of the 4x4 periodic Ising model by enumeration
    g = {}
    for c in range(1 << 16):
        s = np.array([1 if (c >> i) & 1 else -1 for i in range(16)], np.int8)
        P, _, _ = O.observables(s, L)
        g[-P] = g.get(-P, 0) + 1
    bins = (-32, 4, 17)
    walkers = []
    algs = []
    for i in range(4):
        s = gpu.Ising(L)
        gpu.init_(s, "random", rng=gpu.Philox(21, i))
        walkers.append(s)
        algs.append(F.WangLandau(gpu.Philox(21, i), F.WangLandauEnsemble(bins, logf=1.0)))
    stages = F.wang_landau_(walkers, algs, logf_final=2.0 ** -12, flat=0.8, check_sweeps=50,
                            max_sweeps_per_stage=20000)
    assert stages == 13
    centers = -32 + 4 * np.arange(17)
    mask = np.array([c in g for c in centers])
    for a in algs:
        lw = -a.ensemble.logweight  # ln g up to a constant
        est = lw[mask] - lw[mask].max()
        ex = np.log([g[c] for c in centers[mask]])
        ex = ex - ex.max()
        err = est - ex
        assert np.max(np.abs(err)) < 0.5 and np.sqrt(np.mean(err ** 2)) < 0.2, err

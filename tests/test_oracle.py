"""The oracle against the reference's own known answers and golden fixtures (CPU)."""
import json
import math
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_philox_known_answers():
    kat = json.load(open(os.path.join(GOLD, "philox_kat.json")))
    assert len(kat["vectors"]) == 3
    for v in kat["vectors"]:
        assert O.philox(v["ctr"], v["key"]).tolist() == v["out"]
    # published Random123 value for the all-zero input
    assert O.philox([0, 0, 0, 0], [0, 0]).tolist() == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]


def test_site_word_mapping():
    # site i takes word (i>>1)&3 of the call with counter (i>>3, t lo, t hi|colour<<16|purpose<<24, stream)
    for i in (0, 1, 2, 7, 8, 13, 1000):
        for colour in (0, 1):
            w = O.philox([i >> 3, 5, (colour << 16) | (2 << 24), 9], [42, 0])
            assert O.site_word(42, 9, 5, colour, 2, i) == int(w[(i >> 1) & 3])


def test_log_error_bound():
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.random(20000), rng.random(2000) * 1e9, [0.5, 1.0, 2.0, 3.0, 1e-300, 5e-324,
                                                                      2.0 ** -53, 1 - 2.0 ** -53]])
    for x in xs:
        ref = math.log(x)
        got = O.log(x)
        if ref == 0.0:
            assert got == 0.0
        else:
            assert abs(got - ref) <= 2 * math.ulp(ref), (x, got, ref)
    assert O.log(0.0) == -math.inf
    assert math.isnan(O.log(-1.0))


def test_ising_bookkeeping_known_answers():
    # SpinSystems/test/test_ising.jl:8-35 -- 4x4 periodic, all up
    s = np.ones(16, np.int8)
    P, M, Q = O.observables(s, [4, 4])
    assert -P == -32 and M == 16
    s[0] = -1  # flip site 1 (0-based 0): dE = 8
    P2, M2, _ = O.observables(s, [4, 4])
    assert -P2 == -24 and M2 == 14 and (-P2) - (-P) == 8


def test_blume_capel_bookkeeping_known_answers():
    # SpinSystems/test/test_blume_capel.jl:8-31 -- 4x4, J=1, D=0.5, all up: E=-24, M=16
    s = np.ones(16, np.int8)
    P, M, Q = O.observables(s, [4, 4])
    J, D = 1.0, 0.5
    assert -J * P + D * Q == -24.0 and M == 16
    s[0] = 0  # propose 0 at site 1: dpair=-4, dspin=-1, dspin2=-1, dE=3.5
    P2, M2, Q2 = O.observables(s, [4, 4])
    assert P2 - P == -4 and M2 - M == -1 and Q2 - Q == -1
    assert (-J * P2 + D * Q2) - (-J * P + D * Q) == 3.5 and M2 == 15


def test_exact_dos_fixture():
    # SpinSystems/test/test_ising.jl:174-191
    d = json.load(open(os.path.join(GOLD, "ising2d_8x8_logdos.json")))
    tab = dict((e, v) for e, v in d["energy_logdos"])
    assert tab[-128] == math.log(2)
    assert abs(tab[0] - 42.41274640460084) < 1e-12
    assert -124 not in tab
    # the density of states counts all 2^64 configurations
    m = max(tab.values())
    total = m + math.log(sum(math.exp(v - m) for v in tab.values()))
    assert abs(total - 64 * math.log(2)) < 1e-9


def test_tables_match_reference_rules():
    beta = 0.4407
    thr, xm = O.table_ising(2, O.METROPOLIS, beta)
    # a = aligned neighbours; dE = 2*(2a-4); dE <= 0 always accepted
    for up in (0, 1):
        for a in range(5):
            dE = 2 * (2 * a - 4)
            t = int(thr[a + 5 * up])
            if dE <= 0:
                assert t == 2 ** 32
            else:
                assert t == math.floor(math.exp(-beta * dE) * 2 ** 32)
    thr, xm = O.table_ising(2, O.GLAUBER, beta)
    for a in range(5):
        dE = 2 * (2 * a - 4)
        lr = -beta * dE
        p = 1 / (1 + math.exp(-lr)) if lr >= 0 else math.exp(lr) / (1 + math.exp(lr))
        assert int(thr[a]) == math.floor(p * 2 ** 32)
    # heat bath: P(flip) for a down spin with neighbour sum S = p_plus = logistic(2 beta S)
    thr, xm = O.table_ising(2, O.HEATBATH, beta)
    for a in range(5):
        S = 4 - 2 * a  # down spin: aligned a => S = -(2a-4)
        p_plus = 1 / (1 + math.exp(-2 * beta * S)) if S >= 0 else math.exp(2 * beta * S) / (1 + math.exp(2 * beta * S))
        assert int(thr[a]) == math.floor(p_plus * 2 ** 32) and xm[a] == 0
        assert xm[a + 5] == 0xFFFFFFFF


def test_oracle_trajectory_fixture():
    for c in json.load(open(os.path.join(GOLD, "oracle_traj.json"))):
        s = O.init_random(c["model"], c["L"], c["seed"], c["stream"])
        obs, att, acc = O.cb_sweep(s, c["model"], c["L"], c["alg"], c["beta"], c["seed"], stream=c["stream"],
                                   nsweeps=c["nsweeps"], D=c["D"], h=c["h"])
        assert obs.tolist() == c["obs"]
        assert (att, acc) == (c["attempts"], c["accepted"])
        assert s.astype(int).tolist() == c["spins"]


@pytest.mark.parametrize("model,alg", [(O.ISING, O.METROPOLIS), (O.ISING, O.GLAUBER), (O.ISING, O.HEATBATH),
                                       (O.BC, O.METROPOLIS), (O.BC, O.HEATBATH)])
def test_cached_equals_full_after_sweeps(model, alg):
    # SpinSystems/test/test_ising.jl:149-172, test_blume_capel.jl:87-107
    for L in ([6, 8], [4, 4, 4]):
        s = O.init_random(model, L, 7)
        obs, att, acc = O.cb_sweep(s, model, L, alg, 0.4, 7, nsweeps=5, D=0.2, h=0.1)
        assert tuple(obs[-1]) == O.observables(s, L)
        assert att == 5 * int(np.prod(L))


def _exact_energy_dist(beta):
    d = json.load(open(os.path.join(GOLD, "ising2d_8x8_logdos.json")))
    E = np.array([e for e, _ in d["energy_logdos"]], float)
    lw = np.array([v for _, v in d["energy_logdos"]]) - beta * E
    lw -= lw.max()
    p = np.exp(lw)
    return E, p / p.sum()


@pytest.mark.parametrize("mode", ["checkerboard", "sequential"])
def test_energy_distribution_matches_exact_dos(mode):
    """Sampled <E> at L=8, beta=0.4 within 3 sigma (binned errors) of the exact DOS
    (distribution_exact_ising2D, SpinSystems/src/ising2d_exact.jl:35-40)."""
    beta, L = 0.4, [8, 8]
    E, p = _exact_energy_dist(beta)
    exact_mean = float((E * p).sum())
    s = O.init_random(O.ISING, L, 11)
    es = []
    if mode == "checkerboard":
        O.cb_sweep(s, O.ISING, L, O.METROPOLIS, beta, 11, nsweeps=200, record=False)
        obs, _, _ = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, beta, 11, sweep0=200, nsweeps=40000)
        es = -obs[:, 0].astype(float)
    else:
        a = 0
        for k in range(20000):
            O.seq_attempts(s, O.ISING, L, O.METROPOLIS, beta, 11, attempt0=a, nattempts=64)
            a += 64
            if k >= 200:
                es.append(-O.observables(s, L)[0])
        es = np.array(es, float)
    nb = 50
    blocks = es[: len(es) // nb * nb].reshape(nb, -1).mean(axis=1)
    err = blocks.std(ddof=1) / math.sqrt(nb)
    assert abs(blocks.mean() - exact_mean) < 3 * err + 1e-9, (blocks.mean(), exact_mean, err)


def test_muca_weight_update_known_answer():
    # test/test_multicanonical.jl:53-80 (integer counts on the device; log restated)
    lnw = np.zeros(5)
    H = np.array([0, 2, 8, 11, 25], np.int64)
    O.muca_update(lnw, H)
    expect = [0.0] + [-math.log(h) for h in (2, 8, 11, 25)]
    assert np.allclose(lnw, expect, rtol=0, atol=1e-15)


def test_flathist_invariants_and_bounds():
    L = [4, 4]
    # E in [-32, 32] step 4 -> 17 bins
    s = O.init_random(O.ISING, L, 5)
    lnw = np.zeros(17)
    H = np.zeros(17, np.int64)
    rc, obs, st, ac = O.flathist_sweep(s, O.ISING, L, O.MUCA, lnw, H, -32, 4, 0.0, 5, nsweeps=20)
    assert rc == O.OK and st == 20 * 16 and H.sum() == st
    assert ac == st  # flat weights: every move accepted (test_multicanonical.jl:30-34)
    # Wang-Landau decrements the visited bin by logf each step (src/algorithms/wang_landau.jl:29-37)
    lnw = np.zeros(17)
    H = np.zeros(17, np.int64)
    rc, obs, st, ac = O.flathist_sweep(s, O.ISING, L, O.WL, lnw, H, -32, 4, math.log(2), 5, sweep0=20, nsweeps=3)
    assert rc == O.OK and np.allclose(lnw, -math.log(2) * H)
    # out-of-range bins stop the run with the counters unchanged (test_multicanonical.jl:39-43)
    s = np.ones(16, np.int8)  # E = -32; one flip gives -24, outside bins {-32, -28}
    lnw = np.zeros(2)
    H = np.zeros(2, np.int64)
    rc, obs, st, ac = O.flathist_sweep(s, O.ISING, L, O.MUCA, lnw, H, -32, 4, 0.0, 5, nsweeps=1)
    assert rc == O.ERR_RANGE and st == 0 and H.sum() == 0


def test_exchange_known_answers():
    # test/test_parallel_ensembles.jl:189-206: beta 1.0 / 0.5, x_i = 0, x_j = -5 -> lr = 2.5 > 0 accepted
    betas = np.array([1.0, 0.5])
    pos = np.array([0, 1], np.int32)
    steps = np.zeros(1, np.uint64)
    acc = np.zeros(1, np.uint64)
    stage = O.pt_exchange(betas, pos, 0, np.array([0.0, -5.0]), 1, 0, 0, steps, acc)
    assert stage == 1 and steps[0] == 1 and acc[0] == 1 and pos.tolist() == [1, 0]
    # odd stage with two replicas: no pair, only the stage toggles (replica_exchange.jl:158-178)
    stage = O.pt_exchange(betas, pos, stage, np.array([0.0, -5.0]), 1, 0, 1, steps, acc)
    assert stage == 0 and steps[0] == 1
    # reversed energies: lr = -2.5, accepted iff log(U) < -2.5
    pos = np.array([0, 1], np.int32)
    hits = 0
    for t in range(4000):
        steps[:] = 0
        acc[:] = 0
        pos[:] = [0, 1]
        O.pt_exchange(betas, pos, 0, np.array([-5.0, 0.0]), 9, 0, t, steps, acc)
        hits += int(acc[0])
    p = math.exp(-2.5)
    assert abs(hits / 4000 - p) < 4 * math.sqrt(p * (1 - p) / 4000)


def test_wl_flatness():
    H = np.array([10, 9, 8, 0, 10], np.int64)
    vis = np.array([1, 1, 1, 0, 1], np.uint8)
    flat, r = O.wl_flat(H, vis, 0.8)
    assert flat and abs(r - 8 / 9.25) < 1e-15
    flat, r = O.wl_flat(H, np.ones(5, np.uint8), 0.8)
    assert not flat and r == 0.0

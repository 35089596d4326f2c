"""Device checkerboard sweeps against the oracle, bit for bit (GPU)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ALG = {"metropolis": O.METROPOLIS, "glauber": O.GLAUBER, "heatbath": O.HEATBATH}


def _alg(mcx, name, seed, beta, stream=0):
    rng = mcx.Philox(seed, stream)
    return {"metropolis": mcx.Metropolis, "glauber": mcx.Glauber, "heatbath": mcx.HeatBath}[name](rng, beta=beta)


def _run_pair(mcx, model, L, alg, beta, seed=42, stream=0, nsweeps=6, D=0.0, h=0.0, J=1.0, layout="int8",
              init="random"):
    if model == O.ISING:
        sys_ = mcx.Ising(L, J=J, h=h, layout=layout)
    else:
        sys_ = mcx.BlumeCapel(L, J=J, D=D, h=h)
    if init == "random":
        mcx.init_(sys_, "random", rng=mcx.Philox(seed, stream))
        s = O.init_random(model, L, seed, stream)
    else:
        s = np.ones(int(np.prod(L)), np.int8)
    assert np.array_equal(sys_.spins, s)
    a = _alg(mcx, alg, seed, beta, stream)
    obs = mcx.sweep_(sys_, a, nsweeps, record=True)
    oobs, att, acc = O.cb_sweep(s, model, L, ALG[alg], beta, seed, stream=stream, nsweeps=nsweeps, J=J, D=D, h=h)
    return sys_, a, obs, s, oobs, att, acc


ISING_CASES = [
    ([4, 4], "metropolis", 0.4407, 0.0),
    ([6, 8], "glauber", 0.3, 0.0),          # W=3: per-site kernel
    ([8, 8], "heatbath", 0.6, 0.0),         # W=4: 4-site words
    ([16, 12], "metropolis", 0.4407, 0.3),  # field
    ([32, 32], "metropolis", 0.4407, 0.0),  # W=16: 128-bit rows
    ([64, 64], "glauber", 0.4407, 0.0),
    ([64, 48], "heatbath", 0.3, -0.2),
    # 64^2 takes 8-site chunks in the one-block kernel; these run as thread-block clusters
    ([128, 64], "metropolis", 0.4407, 0.0),
    ([128, 128], "heatbath", 0.4407, 0.1),
    ([32, 16, 16], "glauber", 0.22, 0.0),
    ([4, 4, 4], "metropolis", 0.22, 0.0),
    ([24, 24, 24], "metropolis", 0.2216, 0.0),
    ([32, 8, 6], "heatbath", 0.25, 0.1),
    ([16, 16, 16], "glauber", 0.2, 0.0),
    # beta so large that some acceptance thresholds are 0: the 64-bit threshold kernels
    ([32, 32], "metropolis", 3.0, 0.0),
    ([16, 16, 16], "heatbath", 3.0, 0.0),
]


@pytest.mark.parametrize("L,alg,beta,h", ISING_CASES)
def test_ising_parity(gpu, L, alg, beta, h):
    sys_, a, obs, s, oobs, att, acc = _run_pair(gpu, O.ISING, L, alg, beta, h=h)
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert a.steps == att
    assert (a.flips if alg == "heatbath" else a.accepted) == acc
    assert gpu.observables(sys_) == gpu.observables(sys_, full=True)


BC_CASES = [
    ([4, 4], "metropolis", 0.5, 1.0, 0.0),
    ([8, 6], "heatbath", 0.7, 0.5, 0.1),
    ([32, 32], "metropolis", 0.6, 1.0, 0.0),
    ([64, 64], "heatbath", 0.6, 1.0, 0.0),
    ([64, 40], "glauber", 0.45, 0.5, 0.2),
    ([128, 96], "metropolis", 0.6, 1.0, 0.0),  # a thread-block cluster
    ([8, 8, 8], "metropolis", 0.3, 1.0, 0.0),
    ([32, 16, 8], "heatbath", 0.35, 0.7, 0.0),
]


@pytest.mark.parametrize("L,alg,beta,D,h", BC_CASES)
def test_blume_capel_parity(gpu, L, alg, beta, D, h):
    sys_, a, obs, s, oobs, att, acc = _run_pair(gpu, O.BC, L, alg, beta, D=D, h=h)
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert (a.flips if alg == "heatbath" else a.accepted) == acc
    assert gpu.observables(sys_) == gpu.observables(sys_, full=True)


@pytest.mark.parametrize("L,alg", [([128, 128], "metropolis"), ([256, 64], "glauber"), ([128, 8, 8], "heatbath")])
def test_msc64_matches_int8_and_oracle(gpu, L, alg):
    sys_, a, obs, s, oobs, att, acc = _run_pair(gpu, O.ISING, L, alg, 0.4407 if len(L) == 2 else 0.22,
                                                layout="msc64")
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)


@pytest.mark.parametrize("L,beta,h", [([128, 16, 8], 0.22, 0.0), ([256, 32], 0.5, 0.25), ([128, 64], 3.0, 0.0)])
def test_msc64_metropolis_forms(gpu, L, beta, h):
    """MSC64 Metropolis: the rank-form kernel on the packed words (no field; also with
    thresholds of 0 at large beta) and, with a field, the int8 arrays of the lattice
    (unpacked before and packed after the call) against the oracle."""
    sys_, a, obs, s, oobs, att, acc = _run_pair(gpu, O.ISING, L, "metropolis", beta, h=h, layout="msc64")
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert a.accepted == acc


def test_l4096_two_sweeps_bit_exact(gpu):
    """configs: 2-D L=4096, seed 7, Metropolis at beta 0.4407, int8 and MSC64."""
    L = [4096, 4096]
    s0 = O.init_random(O.ISING, L, 7)
    s = s0.copy()
    oobs, _, acc = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.4407, 7, nsweeps=2)
    for layout in ("int8", "msc64"):
        sys_ = gpu.Ising(L, layout=layout)
        gpu.init_(sys_, "random", rng=gpu.Philox(7))
        a = gpu.Metropolis(gpu.Philox(7), beta=0.4407)
        obs = gpu.sweep_(sys_, a, 2, record=True)
        assert np.array_equal(obs, oobs)
        assert a.accepted == acc
        assert np.array_equal(sys_.spins, s)
        sys_.close()


STRIP_CASES = [
    # model, dims, algorithm, beta, D, h: lattices above the one-cluster limit with more rows
    # than threads per chunk column, so each thread carries its neighbour rows over runs of
    # two or more rows; 3-D runs cross planes; 16-, 8- and 4-site chunks; thresholds of 0
    (O.ISING, [64, 24, 3600], "metropolis", 0.2216, 0.0, 0.0),  # 2 chunks per row, Ly = 24
    (O.ISING, [32, 48, 4000], "heatbath", 0.22, 0.0, 0.1),      # 1 chunk per row
    (O.ISING, [64, 6, 12000], "glauber", 0.25, 0.0, 0.0),       # Ly = 6: runs cross a plane every few rows
    (O.ISING, [2048, 2048], "metropolis", 3.0, 0.0, 0.0),       # 64-bit thresholds
    (O.ISING, [1008, 2000], "glauber", 0.4407, 0.0, -0.1),      # W = 504: 8-site chunks
    (O.ISING, [1000, 1200], "heatbath", 0.5, 0.0, 0.0),         # W = 500: 4-site chunks
    (O.BC, [2048, 2048], "metropolis", 0.6, 1.0, 0.0),
    (O.BC, [32, 24, 8000], "heatbath", 0.35, 0.7, 0.1),
    (O.BC, [2000, 2048], "glauber", 0.5, 0.5, 0.0),             # W = 1000: 8-site chunks
]


@pytest.mark.parametrize("model,L,alg,beta,D,h", STRIP_CASES)
def test_strip_walk_parity(gpu, model, L, alg, beta, D, h):
    """The column-strip half-sweep (runs of consecutive rows per thread) against the oracle:
    spins, per-sweep series and counters over three sweeps, bit for bit."""
    sys_, a, obs, s, oobs, att, acc = _run_pair(gpu, model, L, alg, beta, D=D, h=h, seed=13, stream=1, nsweeps=3)
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert (a.flips if alg == "heatbath" else a.accepted) == acc
    sys_.close()


@pytest.mark.parametrize("L,beta,nsweeps", [([2048, 1024], 0.4407, 20), ([128, 64, 80], 0.2216, 16),
                                             ([1024, 544], 3.0, 17)])
def test_int8_calls_on_transient_msc64(gpu, L, beta, nsweeps):
    """Large int8 Ising lattices under Metropolis without a field run calls of 16 sweeps or
    more on a packed 64-sites-per-word copy: spins, series and counters still equal the
    oracle's, and a following heat-bath call (int8 kernels) continues from the unpacked
    state."""
    sys_, a, obs, s, oobs, att, acc = _run_pair(gpu, O.ISING, L, "metropolis", beta, seed=21, stream=2,
                                                nsweeps=nsweeps)
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert a.accepted == acc
    hb = _alg(gpu, "heatbath", 22, beta, 0)
    obs2 = gpu.sweep_(sys_, hb, 3, record=True)
    oobs2, _, acc2 = O.cb_sweep(s, O.ISING, L, O.HEATBATH, beta, 22, stream=0, nsweeps=3)
    assert np.array_equal(obs2, oobs2)
    assert np.array_equal(sys_.spins, s)
    assert hb.flips == acc2
    sys_.close()


def test_packing_switch(gpu):
    """mcx_lattice_set_packing(lat, 0) keeps calls on the int8 kernels: no copy is
    allocated and the results are the same; switching it back on gives the packed path."""
    L = [2048, 1024]
    ctx = gpu.Context()
    sys_ = gpu.Ising(L, ctx=ctx)
    gpu.init_(sys_, "random", rng=gpu.Philox(8))
    sys_.set_packing(False)
    before = ctx.memory()[0]
    a = gpu.Metropolis(gpu.Philox(8), beta=0.4407)
    obs = gpu.sweep_(sys_, a, 16, record=True)
    assert ctx.memory()[0] == before
    s = O.init_random(O.ISING, L, 8)
    oobs, _, acc = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.4407, 8, nsweeps=16)
    assert np.array_equal(obs, oobs) and np.array_equal(sys_.spins, s) and a.accepted == acc
    sys_.set_packing(True)
    obs = gpu.sweep_(sys_, a, 16, record=True)
    assert ctx.memory()[0] == before + L[0] * L[1] // 8
    oobs, _, _ = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.4407, 8, sweep0=16, nsweeps=16)
    assert np.array_equal(obs, oobs) and np.array_equal(sys_.spins, s)
    sys_.close()


def test_transient_msc64_respects_the_budget(gpu):
    """With no room in the HBM budget for the packed copy the call stays on the int8
    kernels, with the same results and no memory taken."""
    L = [4096, 2048]
    probe = gpu.Context()
    lat = gpu.Ising(L, ctx=probe)
    used = probe.memory()[0]
    lat.close()
    probe.close()
    ctx = gpu.Context(hbm_budget=used + (64 << 10))
    sys_ = gpu.Ising(L, ctx=ctx)
    gpu.init_(sys_, "random", rng=gpu.Philox(4))
    before = ctx.memory()[0]
    a = gpu.Metropolis(gpu.Philox(4), beta=0.4407)
    obs = gpu.sweep_(sys_, a, 16, record=True)
    assert ctx.memory()[0] == before
    s = O.init_random(O.ISING, L, 4)
    oobs, _, acc = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.4407, 4, nsweeps=16)
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert a.accepted == acc
    sys_.close()


def test_sweeps_compose_and_replay(gpu):
    """Counter-based stream: 3+5 sweeps equal 8 sweeps; a replay from the same
    counter reproduces the run."""
    L = [64, 32]
    a1 = gpu.Ising(L)
    gpu.init_(a1, "random", rng=gpu.Philox(1))
    m1 = gpu.Metropolis(gpu.Philox(5), beta=0.5)
    gpu.sweep_(a1, m1, 3)
    gpu.sweep_(a1, m1, 5)
    a2 = gpu.Ising(L)
    gpu.init_(a2, "random", rng=gpu.Philox(1))
    m2 = gpu.Metropolis(gpu.Philox(5), beta=0.5)
    gpu.sweep_(a2, m2, 8)
    assert np.array_equal(a1.spins, a2.spins)
    assert m1.accepted == m2.accepted and m1.rng.counter == 8


def test_replayed_sequence_follows_each_calls_stream(gpu):
    """Multi-sweep calls replay one captured sequence per (algorithm, beta, length):
    every replay must still use its own call's seed, stream and counter."""
    L = [1088, 512]  # above the one-cluster limit: captured graph replay
    s0 = O.init_random(O.ISING, L, 1, 0)
    sys_ = gpu.Ising(L)
    for seed, stream, counter in ((11, 0, 0), (12, 3, 0), (11, 0, 40), (99, 7, 5)):
        sys_.spins = s0
        a = gpu.Metropolis(gpu.Philox(seed, stream, counter), beta=0.45)
        obs = gpu.sweep_(sys_, a, 66, record=True)
        s = s0.copy()
        oobs, att, acc = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.45, seed, stream=stream, nsweeps=66,
                                    sweep0=counter)
        assert np.array_equal(obs, oobs), (seed, stream, counter)
        assert np.array_equal(sys_.spins, s)
        assert a.accepted == acc


@pytest.mark.parametrize("model,L,alg,nsweeps", [(O.ISING, [1024, 544], "metropolis", 71),
                                                  (O.BC, [736, 736], "heatbath", 66),
                                                  (O.ISING, [64, 64, 136], "glauber", 65),
                                                  (O.ISING, [130, 256], "metropolis", 65)])  # rows of 65: site kernel
def test_chunked_graph_replay(gpu, model, L, alg, nsweeps):
    """Lattices above the one-cluster limit (and medium ones whose rows are not a multiple
    of four) replay a captured 64-sweep chunk back to back and
    launch the remainder directly; every call (any length, seed, stream, counter) matches
    the oracle, series included."""
    D = 1.0 if model == O.BC else 0.0
    s0 = O.init_random(model, L, 3, 0)
    sys_ = gpu.Ising(L) if model == O.ISING else gpu.BlumeCapel(L, D=D)
    for seed, stream, counter, n in ((5, 0, 0, nsweeps), (6, 2, 17, nsweeps), (5, 1, 3, nsweeps + 64)):
        sys_.spins = s0
        a = _alg(gpu, alg, seed, 0.4 if len(L) == 2 else 0.22, stream)
        a.rng.counter = counter
        obs = gpu.sweep_(sys_, a, n, record=True)
        s = s0.copy()
        oobs, att, acc = O.cb_sweep(s, model, L, ALG[alg], 0.4 if len(L) == 2 else 0.22, seed, stream=stream,
                                    sweep0=counter, nsweeps=n, D=D)
        assert np.array_equal(obs, oobs), (seed, stream, counter, n)
        assert np.array_equal(sys_.spins, s)
        assert (a.flips if alg == "heatbath" else a.accepted) == acc


CLUSTER_CASES = [
    # model, dims, algorithm, beta, D, h: medium lattices (4,096 < N <= 524,288 sites), every
    # sweep of a call in one thread-block cluster; uneven cuts, 4/8/16-site chunks, 3-D planes
    (O.ISING, [256, 256], "metropolis", 0.4407, 0.0, 0.0),
    (O.ISING, [512, 512], "heatbath", 0.44, 0.0, 0.1),
    (O.ISING, [200, 200], "glauber", 0.4, 0.0, 0.0),
    (O.ISING, [4096, 8], "metropolis", 3.0, 0.0, 0.0),  # 8 rows: 8 CTAs; thresholds of 0
    (O.ISING, [64, 64, 16], "metropolis", 0.2216, 0.0, 0.0),
    (O.ISING, [40, 40, 40], "heatbath", 0.22, 0.0, 0.0),
    (O.ISING, [128, 64, 8], "glauber", 0.25, 0.0, -0.2),
    (O.BC, [256, 256], "metropolis", 0.6, 1.0, 0.0),
    (O.BC, [200, 160], "heatbath", 0.5, 0.5, 0.1),
    (O.BC, [32, 32, 32], "metropolis", 0.35, 1.0, 0.0),
    (O.BC, [64, 64, 64], "heatbath", 0.3, 0.7, 0.0),
]


@pytest.mark.parametrize("model,L,alg,beta,D,h", CLUSTER_CASES)
def test_cluster_parity(gpu, model, L, alg, beta, D, h):
    """The cluster form (rows or planes spread over the CTAs' shared memory, halos through
    distributed shared memory) equals the oracle bit for bit: series, spins, counters."""
    sys_, a, obs, s, oobs, att, acc = _run_pair(gpu, model, L, alg, beta, D=D, h=h)
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert a.steps == att
    assert (a.flips if alg == "heatbath" else a.accepted) == acc
    assert gpu.observables(sys_) == gpu.observables(sys_, full=True)


def test_cluster_calls_compose(gpu):
    """Cluster form: 1 + 3 + 70 sweeps equal one call of 74, and the oracle."""
    L = [256, 192]
    s0 = O.init_random(O.ISING, L, 2, 0)
    runs = []
    for parts in ((1, 3, 70), (74,)):
        sys_ = gpu.Ising(L)
        sys_.spins = s0
        a = gpu.Metropolis(gpu.Philox(8, 1), beta=0.42)
        obs = np.concatenate([gpu.sweep_(sys_, a, n, record=True) for n in parts])
        runs.append((obs, sys_.spins.copy(), a.accepted))
    s = s0.copy()
    oobs, att, acc = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.42, 8, stream=1, nsweeps=74)
    for obs, spins, accepted in runs:
        assert np.array_equal(obs, oobs) and np.array_equal(spins, s) and accepted == acc


def test_context_outlives_its_objects(gpu):
    """Destroying the context handle first leaves its lattices usable; the stream and
    accounting go away with the last object (finalisers may run in any order)."""
    ctx = gpu.Context()
    sys_ = gpu.Ising([16, 16], ctx=ctx)
    gpu.init_(sys_, "random", rng=gpu.Philox(3))
    s = O.init_random(O.ISING, [16, 16], 3)
    ctx.close()
    a = gpu.Metropolis(gpu.Philox(3), beta=0.4)
    obs = gpu.sweep_(sys_, a, 3, record=True)
    oobs, _, _ = O.cb_sweep(s, O.ISING, [16, 16], O.METROPOLIS, 0.4, 3, nsweeps=3)
    assert np.array_equal(obs, oobs)
    sys_.close()


def test_known_answers_through_the_abi(gpu):
    # SpinSystems/test/test_ising.jl:8-35
    sys_ = gpu.Ising([4, 4])
    assert gpu.energy(sys_) == -32 and gpu.magnetization(sys_) == 16
    sp = sys_.spins
    sp[0] = -1
    sys_.spins = sp
    assert gpu.energy(sys_) == -24 and gpu.magnetization(sys_) == 14
    # SpinSystems/test/test_blume_capel.jl:8-31
    bc = gpu.BlumeCapel([4, 4], J=1.0, D=0.5)
    assert gpu.energy(bc) == -24.0 and gpu.magnetization(bc) == 16
    sp = bc.spins
    sp[0] = 0
    bc.spins = sp
    assert gpu.energy(bc) == -24.0 + 3.5 and gpu.magnetization(bc) == 15
    gpu.init_(bc, "zero")
    assert gpu.magnetization(bc) == 0 and gpu.energy(bc) == 0.0
    gpu.init_(bc, "down")
    assert np.all(bc.spins == -1)


def test_argument_errors(gpu):
    # the colour-split lattice needs even sides >= 4 (other grids run as general graphs)
    with pytest.raises(gpu.ArgumentError):
        gpu.IsingLatticeOptim(5, 8)
    with pytest.raises(gpu.ArgumentError):
        gpu.IsingDevice([2, 8])
    with pytest.raises(gpu.ArgumentError):
        gpu.Ising([5, 8], layout="msc64")
    with pytest.raises(gpu.ArgumentError):
        gpu.Ising([64, 64], layout="msc64")  # Lx must be a multiple of 128
    sys_ = gpu.Ising([8, 8])
    with pytest.raises(gpu.ArgumentError):
        sys_.spins = np.zeros(64, np.int8)  # 0 is not an Ising state
    with pytest.raises(gpu.ArgumentError):
        gpu.init_(sys_, "zero")
    with pytest.raises(gpu.ArgumentError):
        gpu.init_(sys_, "random")


@pytest.mark.parametrize("L,layout", [([8, 8], "int8"), ([2048, 1024], "int8"), ([128, 64], "msc64")])
def test_sweep_call_edges(gpu, L, layout):
    """Zero sweeps change nothing and return an empty series (on the one-block, packed-copy
    and MSC64 paths); a negative count, a non-finite beta and a sweep counter beyond 2^48 are
    argument errors that leave the lattice and the rng as they were."""
    sys_ = gpu.Ising(L, layout=layout)
    gpu.init_(sys_, "random", rng=gpu.Philox(3))
    s0 = sys_.spins
    e0 = gpu.observables(sys_)
    a = gpu.Metropolis(gpu.Philox(3), beta=0.44)
    obs = gpu.sweep_(sys_, a, 0, record=True)
    assert obs.shape == (0, 3) and a.steps == 0 and a.rng.counter == 0
    assert np.array_equal(sys_.spins, s0) and gpu.observables(sys_) == e0
    with pytest.raises(gpu.ArgumentError):
        gpu.sweep_(sys_, a, -1)
    with pytest.raises(gpu.ArgumentError):
        gpu.sweep_(sys_, gpu.Metropolis(gpu.Philox(3), beta=float("nan")), 1)
    with pytest.raises(gpu.ArgumentError):
        gpu.sweep_(sys_, gpu.Metropolis(gpu.Philox(3, 0, (1 << 48) - 4), beta=0.44), 20)
    assert np.array_equal(sys_.spins, s0) and a.rng.counter == 0
    sys_.close()


def test_hbm_budget(gpu):
    ctx = gpu.Context(hbm_budget=1 << 20)
    with pytest.raises(gpu.BudgetError):
        gpu.Ising([2048, 2048], ctx=ctx)
    small = gpu.Ising([64, 64], ctx=ctx)
    used, budget = ctx.memory()
    assert 0 < used <= budget
    small.close()


@pytest.mark.parametrize("L,alg", [([4096, 64], "metropolis"), ([48, 48, 48], "heatbath"), ([96, 80], "glauber")])
def test_autotune_keeps_results(gpu, L, alg):
    """The autotuner only picks a kernel shape; results stay bit-identical to the oracle."""
    sys_ = gpu.Ising(L)
    gpu.init_(sys_, "random", rng=gpu.Philox(4))
    a = _alg(gpu, alg, 4, 0.3 if len(L) == 2 else 0.22)
    width, ns = gpu.autotune_(sys_, a)
    assert width in (4, 8, 16) and ns > 0
    obs = gpu.sweep_(sys_, a, 3, record=True)
    s = O.init_random(O.ISING, L, 4)
    oobs, _, acc = O.cb_sweep(s, O.ISING, L, ALG[alg], 0.3 if len(L) == 2 else 0.22, 4, nsweeps=3)
    assert np.array_equal(obs, oobs) and np.array_equal(sys_.spins, s)


@pytest.mark.parametrize("model,dims,alg", [
    (O.ISING, [[64, 64], [32, 48], [8, 8], [128, 128], [6, 10]], "metropolis"),
    (O.ISING, [[16, 16, 16], [8, 8, 12]], "heatbath"),
    (O.BC, [[64, 64], [16, 24], [40, 8]], "heatbath"),
    (O.BC, [[32, 32], [8, 8]], "metropolis"),
    (O.ISING, [[64, 64], [256, 128]], "glauber"),   # above the one-block size: one cluster per lattice
    (O.ISING, [[256, 256], [128, 128], [192, 160]], "metropolis"),
    (O.BC, [[256, 256], [256, 256]], "heatbath"),
    (O.ISING, [[32, 32, 32], [64, 64, 16]], "heatbath"),
    (O.ISING, [[32, 32], [1024, 544]], "metropolis"),  # above the one-cluster size: one call each
    (O.ISING, [[128, 128], [128, 64]], "metropolis"),  # a few chains above 4,096 sites: one cluster each
    (O.ISING, [[128, 64]] * 20, "metropolis"),         # more chains than clusters at once: 16-site chunks
    (O.BC, [[96, 96], [128, 128]], "metropolis"),
    (O.ISING, [[64, 64], [128, 128]], "heatbath"),     # 8-site chunks (the narrower lattice's width)
    (O.BC, [[128, 128], [64, 128]], "metropolis"),
    (O.BC, [[64, 64]], "glauber"),                    # 8-site chunks
])
def test_sweep_batch_matches_each_chain(gpu, model, dims, alg):
    """Independent chains in one call (ParallelChains): each lattice's series, spins and
    counters equal its own oracle run."""
    systems, algs, refs = [], [], []
    for i, L in enumerate(dims):
        beta = (0.3 + 0.05 * i) if len(L) == 2 else 0.2 + 0.01 * i
        D = 0.5 + 0.1 * i if model == O.BC else 0.0
        sysd = gpu.Ising(L) if model == O.ISING else gpu.BlumeCapel(L, D=D)
        gpu.init_(sysd, "random", rng=gpu.Philox(10 + i, i))
        a = _alg(gpu, alg, 20 + i, beta, stream=i)
        a.rng.counter = 3 * i
        s = O.init_random(model, L, 10 + i, i)
        refs.append((s, L, beta, D, a.rng.counter))
        systems.append(sysd)
        algs.append(a)
    obs = gpu.sweep_batch_(systems, algs, 25, record=True)
    for i, (s, L, beta, D, c0) in enumerate(refs):
        oobs, att, acc = O.cb_sweep(s, model, L, ALG[alg], beta, 20 + i, stream=i, sweep0=c0, nsweeps=25, D=D)
        assert np.array_equal(obs[i], oobs), (i, L)
        assert np.array_equal(systems[i].spins, s)
        assert algs[i].steps == att and (algs[i].flips if alg == "heatbath" else algs[i].accepted) == acc
        assert algs[i].rng.counter == c0 + 25
        assert gpu.observables(systems[i]) == gpu.observables(systems[i], full=True)


def test_sweep_batch_argument_errors(gpu):
    a = gpu.Ising([8, 8])
    b = gpu.BlumeCapel([8, 8], D=1.0)
    with pytest.raises(gpu.ArgumentError):
        gpu.sweep_batch_([a, b], [gpu.Metropolis(gpu.Philox(1), beta=0.3), gpu.Metropolis(gpu.Philox(2), beta=0.3)], 2)
    with pytest.raises(gpu.ArgumentError):
        gpu.sweep_batch_([a, a], [gpu.Metropolis(gpu.Philox(1), beta=0.3), gpu.HeatBath(gpu.Philox(2), beta=0.3)], 2)

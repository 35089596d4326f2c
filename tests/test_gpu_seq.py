"""spin_flip!(sys, alg) on device systems: the reference's random-site order and FP64
decisions, against the oracle's sequential mode (GPU).  Lattices: bit for bit.  General
graphs: spins, M and counters bit for bit, E within the tolerance written below."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ALG = {"metropolis": O.METROPOLIS, "glauber": O.GLAUBER, "heatbath": O.HEATBATH}

CASES = [
    # model, L, alg, beta, J, D, h, layout
    (O.ISING, [8, 8], "metropolis", 0.4407, 1.0, 0.0, 0.0, "int8"),
    (O.ISING, [16, 12], "glauber", 0.3, 1.0, 0.0, 0.3, "int8"),
    (O.ISING, [8, 8, 8], "heatbath", 0.22, 1.0, 0.0, 0.0, "int8"),
    (O.ISING, [6, 4, 10], "metropolis", 0.5, 0.5, 0.0, -0.2, "int8"),
    (O.ISING, [64, 64], "heatbath", 0.6, 1.0, 0.0, 0.1, "int8"),
    (O.BC, [16, 16], "metropolis", 0.6, 1.0, 1.0, 0.0, "int8"),
    (O.BC, [12, 8], "heatbath", 0.7, 1.0, 0.5, 0.1, "int8"),
    (O.BC, [8, 6, 4], "glauber", 0.35, 1.0, 0.7, 0.0, "int8"),
    # above the shared-memory size: the attempts read and write global memory
    (O.ISING, [512, 512], "metropolis", 0.4407, 1.0, 0.0, 0.0, "int8"),
    (O.BC, [64, 64, 64], "heatbath", 0.4, 1.0, 1.0, 0.0, "int8"),
    # 64 spins per word
    (O.ISING, [128, 128], "glauber", 0.4407, 1.0, 0.0, 0.0, "msc64"),
]


def _system(gpu, model, L, J, D, h, layout):
    if model == O.ISING:
        return gpu.Ising(L, J=J, h=h, layout=layout)
    return gpu.BlumeCapel(L, J=J, D=D, h=h)


@pytest.mark.parametrize("model,L,alg,beta,J,D,h,layout", CASES)
def test_spin_flip_matches_sequential_oracle(gpu, model, L, alg, beta, J, D, h, layout):
    seed, stream = 31, 3
    N = int(np.prod(L))
    n1, n2 = 2 * N + 7, min(N, 50000) + 25  # two calls; the counter carries over
    sys_ = _system(gpu, model, L, J, D, h, layout)
    gpu.init_(sys_, "random", rng=gpu.Philox(seed, stream))
    a = {"metropolis": gpu.Metropolis, "glauber": gpu.Glauber, "heatbath": gpu.HeatBath}[alg](
        gpu.Philox(seed, stream), beta=beta)
    gpu.spin_flip_(sys_, a, n1)
    gpu.spin_flip_(sys_, a, n2)
    s = O.init_random(model, L, seed, stream)
    st, ac = O.seq_attempts(s, model, L, ALG[alg], beta, seed, stream=stream, attempt0=0, nattempts=n1 + n2,
                            J=J, D=D, h=h)
    assert np.array_equal(sys_.spins, s)
    assert a.steps == st == n1 + n2
    assert (a.flips if alg == "heatbath" else a.accepted) == ac
    assert a.rng.counter == n1 + n2
    assert gpu.observables(sys_) == O.observables(s, L)
    assert gpu.observables(sys_) == gpu.observables(sys_, full=True)
    sys_.close()


def test_spin_flip_one_at_a_time_is_the_reference_loop(gpu):
    """`for _ in 1:n; spin_flip!(sys, alg); end` equals one call of n attempts, and a
    sweep_ after spin flips continues the same counter without reusing random words."""
    L = [16, 16]
    a1 = gpu.Ising(L)
    gpu.init_(a1, "random", rng=gpu.Philox(5))
    m1 = gpu.Metropolis(gpu.Philox(9), beta=0.5)
    for _ in range(40):
        gpu.spin_flip_(a1, m1)
    a2 = gpu.Ising(L)
    gpu.init_(a2, "random", rng=gpu.Philox(5))
    m2 = gpu.Metropolis(gpu.Philox(9), beta=0.5)
    gpu.spin_flip_(a2, m2, 40)
    assert np.array_equal(a1.spins, a2.spins)
    assert (m1.steps, m1.accepted, m1.rng.counter) == (m2.steps, m2.accepted, m2.rng.counter)
    assert m1.rng.counter == 40
    gpu.sweep_(a1, m1, 3)
    s = O.init_random(O.ISING, L, 5)
    O.seq_attempts(s, O.ISING, L, O.METROPOLIS, 0.5, 9, nattempts=40)
    O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.5, 9, sweep0=40, nsweeps=3)
    assert np.array_equal(a1.spins, s)
    assert m1.rng.counter == 43


def test_spin_flip_rejects_bad_arguments(gpu):
    sys_ = gpu.Ising([8, 8])
    a = gpu.Metropolis(gpu.Philox(1), beta=0.3)
    with pytest.raises(gpu.ArgumentError):
        gpu.spin_flip_(sys_, a, -1)
    a.ensemble.beta = float("nan")
    with pytest.raises(gpu.ArgumentError):
        gpu.spin_flip_(sys_, a, 1)
    assert a.rng.counter == 0


def _graph_case(name):
    from graph_cases import from_edges, grid_edges, hub_edges, random_edges
    if name == "grid8_ising":
        n, es = grid_edges([8, 8], True)
        return O.Graph(*from_edges(n, es)[:2], J=1.0)
    if name == "gauss_vector_h":
        es = random_edges(2000, 5000, 4)
        rp, col, val = from_edges(2000, es, np.random.default_rng(5).normal(size=len(es)))
        return O.Graph(rp, col, Jv=val, hv=np.random.default_rng(6).normal(size=2000) * 0.5)
    if name == "hub_uniform_h":
        es = hub_edges(1000, 200, 9)
        return O.Graph(*from_edges(1000, es)[:2], J=1.0, h=0.2)
    if name == "bc_grid":
        n, es = grid_edges([12, 10], True)
        return O.BCGraph(*from_edges(n, es)[:2], J=1.0, D=0.5)
    if name == "bc_gauss_vector_h":
        es = random_edges(2500, 6000, 32)
        rp, col, val = from_edges(2500, es, np.random.default_rng(33).normal(size=len(es)))
        return O.BCGraph(rp, col, Jv=val, D=0.3, hv=np.random.default_rng(34).normal(size=2500) * 0.5)
    if name == "bc_open_uniform_h":
        n, es = grid_edges([9, 7], False)
        return O.BCGraph(*from_edges(n, es)[:2], J=1.0, D=1.0, h=0.2)
    raise KeyError(name)


GRAPH_CASES = [("grid8_ising", "metropolis", 0.44), ("gauss_vector_h", "glauber", 0.9),
               ("hub_uniform_h", "heatbath", 0.7), ("bc_grid", "metropolis", 0.6),
               ("bc_gauss_vector_h", "heatbath", 1.0), ("bc_open_uniform_h", "glauber", 0.5)]


@pytest.mark.parametrize("name,alg,beta", GRAPH_CASES)
def test_graph_spin_flip_matches_sequential_oracle(gpu, name, alg, beta):
    """Random-vertex attempts on general graphs: spins, M and counters bit for bit, E within
    1e-12 of the total coupling and field weight (the device's starting E is a recompute
    summed in another order; every later change is the same sequential FP64 sum)."""
    from mcx.graph import BlumeCapelGraphDevice, IsingGraphDevice
    g = _graph_case(name)
    bc = isinstance(g, O.BCGraph)
    h = g.hv if g.hv is not None else g.h
    if bc:
        sysd = BlumeCapelGraphDevice(g.rowptr, g.col, g.Jv, J=g.J, D=g.D, h=h)
        s = O.bcg_init_random(g.n, 8, 1)
    else:
        sysd = IsingGraphDevice(g.rowptr, g.col, g.Jv, J=g.J, h=h)
        s = O.graph_init_random(g.n, 8, 1)
    gpu.init_(sysd, "random", rng=gpu.Philox(8, 1))
    assert np.array_equal(sysd.spins, s)
    a = {"metropolis": gpu.Metropolis, "glauber": gpu.Glauber, "heatbath": gpu.HeatBath}[alg](
        gpu.Philox(12, 4, 100), beta=beta)
    n1, n2 = 3 * g.n + 5, g.n // 2 + 3
    gpu.spin_flip_(sysd, a, n1)
    gpu.spin_flip_(sysd, a, n2)
    E, M, att, acc = O.graph_seq_attempts(g, s, ALG[alg], beta, 12, stream=4, attempt0=100, nattempts=n1 + n2)
    assert np.array_equal(sysd.spins, s)
    assert gpu.magnetization(sysd) == M == gpu.magnetization(sysd, full=True)
    wt = 1.0 + (np.abs(g.Jv).sum() if g.Jv is not None else abs(g.J) * g.col.size) + \
        (np.abs(g.hv).sum() if g.hv is not None else abs(g.h) * g.n)
    assert abs(gpu.energy(sysd) - E) <= 1e-12 * wt
    assert a.steps == att == n1 + n2 and (a.flips if alg == "heatbath" else a.accepted) == acc
    assert a.rng.counter == 100 + n1 + n2
    sysd.close()

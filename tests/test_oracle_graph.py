"""The general-graph oracle (IsingGraph / IsingMatrix) against the reference's known
answers, the exact 8x8 density of states and its own invariants (CPU)."""
import json
import math
import os

import numpy as np
import pytest

import oracle as O
from graph_cases import from_edges, grid_edges, hub_edges, random_edges

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_exp_and_logistic_error_bounds():
    rng = np.random.default_rng(5)
    xs = np.concatenate([rng.uniform(-745, 709, 20000), rng.uniform(-40, 0, 20000), -np.logspace(-300, 2, 2000),
                         [0.0, -0.0, 1.0, -1.0, 0.5, 700.0, -700.0]])
    for x in xs:
        ref = math.exp(x)
        assert abs(O.exp(x) - ref) <= math.ulp(ref), x
    assert O.exp(710.0) == math.inf and O.exp(-746.0) == 0.0 and math.isnan(O.exp(math.nan))
    # test/test_utils.jl:56-67
    assert O.logistic(0.0) == 0.5
    for x in (0.1, 1.0, 5.0, 40.0):
        assert abs(O.logistic(x) + O.logistic(-x) - 1.0) < 1e-15


def _ring4(vals):
    # J[1,2]=J[2,1]=a, J[2,3]=b, J[3,4]=c, J[4,1]=d (0-based here)
    return from_edges(4, [(0, 1), (1, 2), (2, 3), (0, 3)], vals)


def test_sparse_coupling_known_answers():
    # SpinSystems/test/test_ising.jl:36-66
    rp, col, val = _ring4([1.0, 2.0, 3.0, 4.0])
    g = O.Graph(rp, col, Jv=val)
    s = np.ones(4, np.int8)
    assert O.graph_observables(g, s) == (-10.0, 4)
    dE = O.graph_delta_energy(g, s, 0)
    assert dE == 10.0
    s[0] = -1
    E, M = O.graph_observables(g, s)
    assert E == 0.0 and M == 2


def test_field_known_answers():
    # SpinSystems/test/test_ising.jl:68-79: 2x2 periodic grid (a ring of 2 per axis)
    n, es = grid_edges([2, 2], True)
    rp, col, _ = from_edges(n, es)
    s = np.array([1, -1, -1, 1], np.int8)
    g = O.Graph(rp, col, J=1.0, h=0.5)
    pair = sum(int(s[v]) * int(s[u]) for v in range(n) for u in col[rp[v]:rp[v + 1]]) / 2
    assert O.graph_observables(g, s)[0] == -pair - 0.5 * s.sum()
    h_i = np.array([1.0, -1.0, 0.5, 0.0])
    g2 = O.Graph(rp, col, J=1.0, hv=h_i)
    assert O.graph_observables(g2, s)[0] == -pair - float((h_i * s).sum())


def _cases():
    n, es = grid_edges([8, 8], True)
    yield "grid8", O.Graph(*from_edges(n, es)[:2], J=1.0)
    n, es = grid_edges([7, 5], False)
    yield "open7x5_h", O.Graph(*from_edges(n, es)[:2], J=1.0, h=0.3)
    es = random_edges(400, 900, 1)
    vals = np.random.default_rng(2).normal(size=len(es))
    rp, col, val = from_edges(400, es, vals)
    yield "random_gauss", O.Graph(rp, col, Jv=val, hv=np.random.default_rng(3).normal(size=400) * 0.3)
    es = hub_edges(300, 120, 4)
    rp, col, val = from_edges(300, es, np.random.default_rng(5).choice([-1.0, 1.0], len(es)))
    yield "hub_pm", O.Graph(rp, col, Jv=val)


@pytest.mark.parametrize("name,g", list(_cases()))
def test_colouring_is_proper_first_fit(name, g):
    c, ncol = O.graph_colour(g)
    for v in range(g.n):
        nb = g.col[g.rowptr[v]:g.rowptr[v + 1]]
        assert all(c[u] != c[v] for u in nb if u != v)
        lower = {int(c[u]) for u in nb if u < v}
        assert c[v] == min(set(range(len(lower) + 1)) - lower)
    assert ncol == c.max() + 1


@pytest.mark.parametrize("alg", [O.METROPOLIS, O.GLAUBER, O.HEATBATH])
@pytest.mark.parametrize("name,g", list(_cases()))
def test_cached_equals_full_after_sweeps(name, g, alg):
    # SpinSystems/test/test_ising.jl:149-172 on the graph systems
    s = O.graph_init_random(g.n, 9)
    Es, Ms, att, acc = O.graph_sweep(g, s, alg, 0.7, 9, nsweeps=6)
    E, M = O.graph_observables(g, s)
    scale = 1.0 + (np.abs(g.Jv).sum() if g.Jv is not None else g.col.size) + (
        np.abs(g.hv).sum() if g.hv is not None else abs(g.h) * g.n)
    assert abs(Es[-1] - E) <= 1e-12 * scale and Ms[-1] == M
    assert att == 6 * g.n and 0 < acc < att


def test_sweep_order_is_colour_classes():
    """Colour-class order: the l-th site of class c uses words 2b, 2b+1 (b = (l>>5)&1) of
    Philox block B_c + 32 (l>>6) + (l&31); recomputing one sweep by hand agrees."""
    n, es = grid_edges([16, 12], True)
    rp, col, _ = from_edges(n, es)
    g = O.Graph(rp, col, J=1.0, h=0.2)
    s0 = O.graph_init_random(n, 3)
    s = s0.copy()
    O.graph_sweep(g, s, O.METROPOLIS, 0.5, 21, stream=2, sweep0=5, nsweeps=1)
    c, ncol = O.graph_colour(g)
    t = s0.copy()
    visits, Bc = [], 0
    for k in range(ncol):
        members = [v for v in range(n) if c[v] == k]
        visits += [(v, Bc + 32 * (l >> 6) + (l & 31), 2 * ((l >> 5) & 1)) for l, v in enumerate(members)]
        Bc += 32 * ((len(members) + 63) // 64)
    for v, blk, b in visits:
        w = O.philox([blk, 5, 7 << 24, 2], [21, 0])
        u = ((int(w[b]) << 21) | (int(w[b + 1]) >> 11)) * 2.0 ** -53
        dE = O.graph_delta_energy(g, t, v)
        lr = -0.5 * dE
        if lr > 0 or u < O.exp(lr):
            t[v] = -t[v]
    assert np.array_equal(s, t)


def test_graph_energy_distribution_matches_exact_dos():
    """The 8x8 periodic grid as a general graph: <E> at beta=0.4 within 3 sigma of the
    exact density of states (SpinSystems/data/exact_solutions/ising2D_8x8.csv)."""
    d = json.load(open(os.path.join(GOLD, "ising2d_8x8_logdos.json")))
    E = np.array([e for e, _ in d["energy_logdos"]], float)
    lw = np.array([v for _, v in d["energy_logdos"]]) - 0.4 * E
    p = np.exp(lw - lw.max())
    exact = float((E * p).sum() / p.sum())
    n, es = grid_edges([8, 8], True)
    g = O.Graph(*from_edges(n, es)[:2], J=1.0)
    s = O.graph_init_random(n, 13)
    O.graph_sweep(g, s, O.METROPOLIS, 0.4, 13, nsweeps=200)
    Es, _, _, _ = O.graph_sweep(g, s, O.METROPOLIS, 0.4, 13, sweep0=200, nsweeps=40000)
    nb = 50
    blocks = Es[: len(Es) // nb * nb].reshape(nb, -1).mean(axis=1)
    err = blocks.std(ddof=1) / math.sqrt(nb)
    assert abs(blocks.mean() - exact) < 3 * err, (blocks.mean(), exact, err)


def test_grid_graph_restatement(mcxlib):
    """The mirror's Graphs.grid restatement: vertex order, neighbour sets, edge order."""
    G = __import__("mcx.graph", fromlist=["grid"])
    for dims, per in (([4, 3], True), ([5, 2, 3], False), ([2, 2], True), ([1, 6], True), ([7], True)):
        g = G.grid(dims, periodic=per)
        n, es = grid_edges(dims, per)
        assert G.nv(g) == n and G.edges(g) == es and G.ne(g) == len(es)
        rp, col = G.graph_csr(g)
        rp2, col2, _ = from_edges(n, es)
        assert np.array_equal(rp, rp2) and np.array_equal(col, col2)
    g = G.grid([2, 2], periodic=True)
    Jvec = np.arange(1.0, G.ne(g) + 1)
    A = G.matrix_from_edges(g, Jvec)
    assert (A != A.T).nnz == 0 and A.nnz == 2 * G.ne(g)
    with pytest.raises(mcxlib.ArgumentError):
        G.matrix_from_edges(g, Jvec[:-1])


def test_blume_capel_graph_known_answers():
    # SpinSystems/test/test_blume_capel.jl:8-31 on the 4x4 torus as a graph
    n, es = grid_edges([4, 4], True)
    rp, col, _ = from_edges(n, es)
    g = O.BCGraph(rp, col, J=1.0, D=0.5)
    s = np.ones(16, np.int8)
    assert O.bcg_observables(g, s) == (-24.0, 16)
    assert O.bcg_delta_energy(g, s, 0, 0) == 3.5
    s[0] = 0
    assert O.bcg_observables(g, s) == (-24.0 + 3.5, 15)
    assert O.bcg_observables(g, np.zeros(16, np.int8)) == (0.0, 0)


@pytest.mark.parametrize("alg", [O.METROPOLIS, O.GLAUBER, O.HEATBATH])
def test_blume_capel_graph_cached_equals_full(alg):
    es = random_edges(300, 700, 21)
    rp, col, val = from_edges(300, es, np.random.default_rng(22).normal(size=len(es)))
    for g in (O.BCGraph(rp, col, Jv=val, D=0.3, hv=np.random.default_rng(23).normal(size=300) * 0.2),
              O.BCGraph(rp, col, J=1.0, D=0.7, h=0.1)):
        s = O.bcg_init_random(g.n, 4)
        assert set(np.unique(s)) <= {-1, 0, 1} and len(np.unique(s)) == 3
        Es, Ms, att, acc = O.bcg_sweep(g, s, alg, 0.8, 4, nsweeps=5)
        E, M = O.bcg_observables(g, s)
        assert abs(Es[-1] - E) < 1e-9 and Ms[-1] == M and 0 < acc < att


def test_blume_capel_graph_heat_bath_distribution():
    """The three-state heat bath on a graph with no edges samples each site from
    exp(-beta (D s^2 - h s)) / Z (blume_capel.jl:61-85)."""
    n = 4000
    g = O.BCGraph(np.zeros(n + 1, np.int64), np.zeros(0, np.int32), J=1.0, D=0.4, h=0.3)
    s = O.bcg_init_random(n, 8)
    O.bcg_sweep(g, s, O.HEATBATH, 1.0, 8, nsweeps=3)
    w = np.array([math.exp(-1.0 * (0.4 * v * v - 0.3 * v)) for v in (-1, 0, 1)])
    p = w / w.sum()
    counts = np.array([(s == v).sum() for v in (-1, 0, 1)])
    assert np.all(np.abs(counts / n - p) < 4 * np.sqrt(p * (1 - p) / n)), (counts / n, p)


@pytest.mark.parametrize("model,alg,beta,D,h", [(O.ISING, O.METROPOLIS, 0.44, 0.0, 0.0),
                                                 (O.ISING, O.HEATBATH, 0.3, 0.0, 0.2),
                                                 (O.BC, O.METROPOLIS, 0.6, 1.0, 0.0),
                                                 (O.BC, O.HEATBATH, 0.5, 0.5, 0.1)])
def test_graph_sequential_mode_equals_lattice_sequential_mode(model, alg, beta, D, h):
    """On a periodic torus the graph oracle's random-vertex attempts (exp of the library's
    own) and the lattice oracle's (exp of the C library) pick the same sites and take the
    same decisions: the two exps differ by at most an ulp, far below 1 in 10^5 attempts."""
    L = [12, 10]
    n, es = grid_edges(L, True)
    rp, col, _ = from_edges(n, es)
    g = O.BCGraph(rp, col, J=1.0, D=D, h=h) if model == O.BC else O.Graph(rp, col, J=1.0, h=h)
    s1 = O.init_random(model, L, 3)
    s2 = s1.copy()
    st, ac = O.seq_attempts(s1, model, L, alg, beta, 9, stream=2, attempt0=5, nattempts=100000, J=1.0, D=D, h=h)
    E, M, att, acc = O.graph_seq_attempts(g, s2, alg, beta, 9, stream=2, attempt0=5, nattempts=100000)
    assert np.array_equal(s1, s2)
    assert (st, ac) == (att, acc)

"""General graphs and couplings on the device against the oracle (GPU): spins, accepted
counts and magnetizations bit for bit; FP64 energies within a tolerance written below
(the device sums per-block partials in a different order than the oracle's sequential
sum).  Graphs up to 8192 padded sites run in the one-block kernel, larger ones one launch
per colour class; the cases cover both."""
import numpy as np
import pytest

import oracle as O
from graph_cases import from_edges, grid_edges, hub_edges, random_edges

pytestmark = pytest.mark.gpu

ALG = {"metropolis": O.METROPOLIS, "glauber": O.GLAUBER, "heatbath": O.HEATBATH}


def _alg(mcx, name, seed, beta, stream=0, counter=0):
    rng = mcx.Philox(seed, stream, counter)
    return {"metropolis": mcx.Metropolis, "glauber": mcx.Glauber, "heatbath": mcx.HeatBath}[name](rng, beta=beta)


def _scale(g):
    j = np.abs(g.Jv).sum() if g.Jv is not None else abs(g.J) * g.col.size
    h = np.abs(g.hv).sum() if g.hv is not None else abs(g.h) * g.n
    return 1.0 + j + h


# energy tolerance: 1e-12 of the total |coupling| + |field| weight (FP64 summation order)
E_RTOL = 1e-12


def _case(name):
    rng = np.random.default_rng(abs(hash(name)) % 2 ** 32)
    if name == "grid8_graph":
        n, es = grid_edges([8, 8], True)
        return O.Graph(*from_edges(n, es)[:2], J=1.0)
    if name == "open7x5_uniform_h":
        n, es = grid_edges([7, 5], False)
        return O.Graph(*from_edges(n, es)[:2], J=1.0, h=0.3)
    if name == "cube6_vector_h":
        n, es = grid_edges([6, 6, 6], True)
        return O.Graph(*from_edges(n, es)[:2], J=0.7, hv=np.random.default_rng(1).normal(size=n) * 0.5)
    if name == "random_gauss":
        es = random_edges(3000, 6000, 2)
        rp, col, val = from_edges(3000, es, np.random.default_rng(3).normal(size=len(es)))
        return O.Graph(rp, col, Jv=val)
    if name == "random_gauss_h":
        es = random_edges(2000, 5000, 4)
        rp, col, val = from_edges(2000, es, np.random.default_rng(5).normal(size=len(es)))
        return O.Graph(rp, col, Jv=val, h=0.2)
    if name == "hub_pm_vector_h":
        es = hub_edges(1000, 200, 6)
        rp, col, val = from_edges(1000, es, np.random.default_rng(7).choice([-1.0, 1.0], len(es)))
        return O.Graph(rp, col, Jv=val, hv=np.random.default_rng(8).normal(size=1000))
    if name == "hub_graph":
        es = hub_edges(1000, 200, 9)
        return O.Graph(*from_edges(1000, es)[:2], J=1.0)
    if name == "random_big_vector_h":  # above the one-block limit: one launch per class
        es = random_edges(20000, 50000, 11)
        rp, col, val = from_edges(20000, es, np.random.default_rng(12).normal(size=len(es)))
        return O.Graph(rp, col, Jv=val, hv=np.random.default_rng(13).normal(size=20000) * 0.5)
    if name == "grid_big_uniform_h":
        n, es = grid_edges([128, 96], True)
        return O.Graph(*from_edges(n, es)[:2], J=1.0, h=0.1)
    if name == "ea_256":
        n, es = grid_edges([256, 256], True)
        rp, col, val = from_edges(n, es, np.random.default_rng(10).normal(size=len(es)))
        return O.Graph(rp, col, Jv=val)
    raise KeyError(name)


def _device(mcx, g):
    from mcx.graph import IsingGraphDevice
    h = g.hv if g.hv is not None else g.h
    return IsingGraphDevice(g.rowptr, g.col, g.Jv, J=g.J, h=h)


CASES = [("grid8_graph", "metropolis", 0.44), ("grid8_graph", "heatbath", 0.6),
         ("open7x5_uniform_h", "glauber", 0.5), ("cube6_vector_h", "heatbath", 0.3),
         ("cube6_vector_h", "metropolis", 0.25), ("random_gauss", "metropolis", 1.2),
         ("random_gauss", "glauber", 0.8), ("random_gauss_h", "heatbath", 1.0),
         ("hub_pm_vector_h", "metropolis", 0.9), ("hub_graph", "glauber", 0.4), ("hub_graph", "heatbath", 2.0),
         ("random_big_vector_h", "heatbath", 1.1), ("random_big_vector_h", "metropolis", 0.7),
         ("grid_big_uniform_h", "glauber", 0.44)]


@pytest.mark.parametrize("name,alg,beta", CASES)
def test_graph_parity(gpu, name, alg, beta):
    g = _case(name)
    sysd = _device(gpu, g)
    gpu.init_(sysd, "random", rng=gpu.Philox(31, 2))
    s = O.graph_init_random(g.n, 31, 2)
    assert np.array_equal(sysd.spins, s)
    c, ncol = O.graph_colour(g)
    assert np.array_equal(sysd.colours, c) and sysd.info()["colours"] == ncol
    a = _alg(gpu, alg, 17, beta, stream=3, counter=11)
    Es, Ms = gpu.sweep_(sysd, a, 7, record=True)
    oE, oM, att, acc = O.graph_sweep(g, s, ALG[alg], beta, 17, stream=3, sweep0=11, nsweeps=7)
    assert np.array_equal(sysd.spins, s)
    assert np.array_equal(Ms, oM)
    assert np.allclose(Es, oE, rtol=0, atol=E_RTOL * _scale(g))
    assert a.steps == att and (a.flips if alg == "heatbath" else a.accepted) == acc
    assert a.rng.counter == 18
    Ef = gpu.energy(sysd, full=True)
    assert abs(Ef - O.graph_observables(g, s)[0]) <= E_RTOL * _scale(g)
    assert gpu.magnetization(sysd) == gpu.magnetization(sysd, full=True) == oM[-1]
    sysd.close()


def test_edwards_anderson_256(gpu):
    """2-D +-Gaussian spin glass on a 256x256 torus (IsingMatrix), 3 Metropolis sweeps."""
    g = _case("ea_256")
    sysd = _device(gpu, g)
    gpu.init_(sysd, "random", rng=gpu.Philox(5))
    s = O.graph_init_random(g.n, 5)
    a = _alg(gpu, "metropolis", 6, 1.0)
    Es, Ms = gpu.sweep_(sysd, a, 3, record=True)
    oE, oM, att, acc = O.graph_sweep(g, s, O.METROPOLIS, 1.0, 6, nsweeps=3)
    assert np.array_equal(sysd.spins, s) and np.array_equal(Ms, oM) and a.accepted == acc
    assert np.allclose(Es, oE, rtol=0, atol=E_RTOL * _scale(g))


def test_table_and_fp64_paths_agree(gpu):
    """One coupling (integer thresholds per (s, lpi)) and the same coupling written per
    entry (FP64 sums and exp per site) follow the same FP64 rule: identical runs."""
    n, es = grid_edges([12, 10], True)
    rp, col, _ = from_edges(n, es)
    from mcx.graph import IsingGraphDevice
    for alg in ("metropolis", "glauber", "heatbath"):
        out = []
        for coupling in (None, np.ones(col.size)):
            d = IsingGraphDevice(rp, col, coupling, J=1.0, h=0.25)
            gpu.init_(d, "random", rng=gpu.Philox(2))
            a = _alg(gpu, alg, 3, 0.45)
            Es, Ms = gpu.sweep_(d, a, 5, record=True)
            out.append((d.spins, Es, Ms))
            d.close()
        assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][2], out[1][2])
        assert np.allclose(out[0][1], out[1][1], rtol=0, atol=1e-9)


def test_reference_known_answers(gpu):
    # SpinSystems/test/test_ising.jl:36-66 (sparse J), :68-79 (fields), :81-119 (constructors)
    import scipy.sparse as sp
    from mcx import graph as G
    J = sp.lil_matrix((4, 4))
    J[0, 1] = J[1, 0] = 1.0
    J[1, 2] = J[2, 1] = 2.0
    J[2, 3] = J[3, 2] = 3.0
    J[3, 0] = J[0, 3] = 4.0
    sysd = gpu.Ising(J.tocsr())
    assert sysd.kind == "IsingMatrix"
    assert gpu.energy(sysd) == -10.0 and gpu.energy(sysd, full=True) == -10.0 and gpu.magnetization(sysd) == 4
    assert G.delta_energy(sysd, 0) == 10.0
    G.modify_(sysd, 0)
    assert gpu.energy(sysd) == 0.0 and gpu.energy(sysd, full=True) == 0.0 and gpu.magnetization(sysd) == 2
    Jbad = sp.lil_matrix((3, 3))
    Jbad[0, 1] = 1.0
    Jbad[1, 0] = 0.5
    with pytest.raises(gpu.ArgumentError):
        gpu.Ising(Jbad.tocsr())
    # fields
    s = np.array([1, -1, -1, 1], np.int8)
    for h in (0.5, np.array([1.0, -1.0, 0.5, 0.0])):
        d = gpu.Ising([2, 2], J=1.0, h=h)
        d.spins = s
        g = O.Graph(*from_edges(*grid_edges([2, 2], True))[:2], J=1.0,
                    **({"h": h} if np.isscalar(h) else {"hv": h}))
        assert gpu.energy(d) == O.graph_observables(g, s)[0] == gpu.energy(d, full=True)
    # constructor variants
    assert gpu.Ising([2, 2], J=1).kind == "IsingGraph"
    assert gpu.Ising([2, 2], J=1, h=np.array([0.1, -0.2, 0.3, 0.0])).kind == "IsingGraph"
    grid = G.grid([2, 2], periodic=True)
    Jvec = np.arange(1.0, G.ne(grid) + 1)
    assert gpu.Ising(grid, Jvec).kind == "IsingMatrix"
    assert gpu.Ising([2, 2], J=Jvec, periodic=True).kind == "IsingMatrix"
    with pytest.raises(gpu.ArgumentError):
        gpu.Ising(grid, Jvec[:-1])
    # grids the colour-split lattice does not take run as graphs
    for dims, per in (([5, 8], True), ([6, 6], False), ([10], True)):
        d = gpu.Ising(dims, periodic=per)
        n, es = grid_edges(dims, per)
        assert gpu.energy(d) == -len(es) and gpu.magnetization(d) == n


def test_graph_errors(gpu):
    from mcx.graph import IsingGraphDevice
    rp, col, _ = from_edges(4, [(0, 1), (1, 2)])
    with pytest.raises(gpu.ArgumentError):
        IsingGraphDevice(rp, col[::-1].copy())  # rows not increasing / not symmetric
    with pytest.raises(gpu.ArgumentError):
        IsingGraphDevice(rp, np.array([1, 0, 2, 9], np.int32))  # out of range
    d = IsingGraphDevice(rp, col)
    with pytest.raises(gpu.ArgumentError):
        d.spins = np.array([1, 0, 1, 1], np.int8)
    assert np.array_equal(d.spins, np.ones(4, np.int8))  # nothing stored
    with pytest.raises(gpu.BoundsError):
        __import__("mcx.graph", fromlist=["x"]).delta_energy(d, 4)
    with pytest.raises(gpu.ArgumentError):
        gpu.init_(d, "zero")


# ---------------------------------------------------------------- Blume-Capel --
def _bc_case(name):
    if name == "bc_grid8":
        n, es = grid_edges([8, 8], True)
        return O.BCGraph(*from_edges(n, es)[:2], J=1.0, D=0.5)
    if name == "bc_open7x5_uniform_h":
        n, es = grid_edges([7, 5], False)
        return O.BCGraph(*from_edges(n, es)[:2], J=1.0, D=1.0, h=0.2)
    if name == "bc_random_gauss_vector_h":
        es = random_edges(2500, 6000, 31)
        rp, col, val = from_edges(2500, es, np.random.default_rng(32).normal(size=len(es)))
        return O.BCGraph(rp, col, Jv=val, D=0.3, hv=np.random.default_rng(33).normal(size=2500) * 0.5)
    if name == "bc_hub":
        es = hub_edges(1000, 150, 34)
        return O.BCGraph(*from_edges(1000, es)[:2], J=0.5, D=0.2)
    if name == "bc_cube_vector_h":  # one J, a field per site: FP64 path
        n, es = grid_edges([6, 6, 6], True)
        return O.BCGraph(*from_edges(n, es)[:2], J=1.0, D=0.6, hv=np.random.default_rng(35).normal(size=n))
    if name == "bc_big_table":  # above the one-block limit
        n, es = grid_edges([120, 100], False)
        return O.BCGraph(*from_edges(n, es)[:2], J=1.0, D=1.0, h=0.05)
    if name == "bc_big_gauss":
        es = random_edges(12000, 30000, 36)
        rp, col, val = from_edges(12000, es, np.random.default_rng(37).normal(size=len(es)))
        return O.BCGraph(rp, col, Jv=val, D=0.5)
    raise KeyError(name)


BC_CASES = [("bc_grid8", "metropolis", 0.6), ("bc_grid8", "heatbath", 0.6), ("bc_open7x5_uniform_h", "glauber", 0.5),
            ("bc_random_gauss_vector_h", "metropolis", 1.0), ("bc_random_gauss_vector_h", "heatbath", 1.0),
            ("bc_hub", "glauber", 0.7), ("bc_hub", "heatbath", 1.5), ("bc_cube_vector_h", "heatbath", 0.4),
            ("bc_big_table", "metropolis", 0.6), ("bc_big_table", "heatbath", 0.6), ("bc_big_gauss", "glauber", 1.2)]


@pytest.mark.parametrize("name,alg,beta", BC_CASES)
def test_blume_capel_graph_parity(gpu, name, alg, beta):
    from mcx.graph import BlumeCapelGraphDevice
    g = _bc_case(name)
    sysd = BlumeCapelGraphDevice(g.rowptr, g.col, g.Jv, J=g.J, D=g.D, h=g.hv if g.hv is not None else g.h)
    gpu.init_(sysd, "random", rng=gpu.Philox(41, 1))
    s = O.bcg_init_random(g.n, 41, 1)
    assert np.array_equal(sysd.spins, s)
    a = _alg(gpu, alg, 43, beta, stream=2, counter=7)
    Es, Ms = gpu.sweep_(sysd, a, 6, record=True)
    oE, oM, att, acc = O.bcg_sweep(g, s, ALG[alg], beta, 43, stream=2, sweep0=7, nsweeps=6)
    assert np.array_equal(sysd.spins, s)
    assert np.array_equal(Ms, oM)
    scale = _scale(g) + abs(g.D) * g.n
    assert np.allclose(Es, oE, rtol=0, atol=E_RTOL * scale)
    assert (a.flips if alg == "heatbath" else a.accepted) == acc
    assert abs(gpu.energy(sysd, full=True) - O.bcg_observables(g, s)[0]) <= E_RTOL * scale


def test_blume_capel_graph_known_answers(gpu):
    # SpinSystems/test/test_blume_capel.jl:8-31 on graphs; constructors blume_capel.jl:467-511
    import scipy.sparse as sp
    from mcx import graph as G
    d = gpu.BlumeCapel([5, 5], D=0.5)  # odd sides: a BlumeCapelGraph on the torus
    assert d.kind == "BlumeCapelGraph"
    n, es = grid_edges([5, 5], True)
    assert gpu.energy(d) == -len(es) + 0.5 * n and gpu.magnetization(d) == n
    g = O.BCGraph(*from_edges(n, es)[:2], J=1.0, D=0.5)
    s = np.ones(n, np.int8)
    assert G.delta_energy(d, 0, 0) == O.bcg_delta_energy(g, s, 0, 0)
    G.modify_(d, 0, 0)
    s[0] = 0
    assert gpu.energy(d) == O.bcg_observables(g, s)[0] == gpu.energy(d, full=True)
    assert gpu.magnetization(d) == n - 1
    gpu.init_(d, "zero")
    assert gpu.energy(d) == 0.0 and gpu.magnetization(d) == 0
    grid = G.grid([3, 4], periodic=False)
    assert gpu.BlumeCapel(grid, 1.0, 0.5).kind == "BlumeCapelGraph"
    Jvec = np.arange(1.0, G.ne(grid) + 1)
    assert gpu.BlumeCapel(grid, Jvec, 0.5).kind == "BlumeCapelMatrix"
    assert gpu.BlumeCapel(sp.csr_matrix(G.matrix_from_edges(grid, Jvec)), 0.5).kind == "BlumeCapelMatrix"
    assert gpu.BlumeCapel([6, 6], periodic=False, D=1.0).kind == "BlumeCapelGraph"
    with pytest.raises(gpu.ArgumentError):
        G.delta_energy(d, 0)  # a Blume-Capel site needs the new state
    with pytest.raises(gpu.ArgumentError):
        d.spins = np.full(n, 2, np.int8)


@pytest.mark.parametrize("bc", [False, True])
def test_graph_edge_cases(gpu, bc):
    """One site, no edges, J = 0, beta = 0: the paths still agree with the oracle."""
    from mcx.graph import IsingGraphDevice, BlumeCapelGraphDevice
    cases = [(np.array([0, 0], np.int64), np.zeros(0, np.int32), None, 1.0, 0.0),     # one site
             (np.zeros(101, np.int64), np.zeros(0, np.int32), None, 1.0, 0.3),       # 100 isolated sites, field
             (*from_edges(50, random_edges(50, 80, 51))[:2], None, 0.0, 0.0),        # J = 0
             (*from_edges(60, random_edges(60, 90, 52), np.zeros(90)), 1.0, 0.2)]    # per-entry zeros
    for rp, col, jv, J, h in cases:
        n = len(rp) - 1
        for alg, beta in (("metropolis", 0.0), ("heatbath", 0.7), ("glauber", 1.3)):
            if bc:
                g = O.BCGraph(rp, col, Jv=jv, J=J, D=0.4, h=h)
                d = BlumeCapelGraphDevice(rp, col, jv, J=J, D=0.4, h=h)
                s = O.bcg_init_random(n, 9)
                gpu.init_(d, "random", rng=gpu.Philox(9))
            else:
                g = O.Graph(rp, col, Jv=jv, J=J, h=h)
                d = IsingGraphDevice(rp, col, jv, J=J, h=h)
                s = O.graph_init_random(n, 9)
                gpu.init_(d, "random", rng=gpu.Philox(9))
            a = _alg(gpu, alg, 3, beta)
            Es, Ms = gpu.sweep_(d, a, 4, record=True)
            sweep = O.bcg_sweep if bc else O.graph_sweep
            oE, oM, att, acc = sweep(g, s, ALG[alg], beta, 3, nsweeps=4)
            assert np.array_equal(d.spins, s) and np.array_equal(Ms, oM), (n, alg, beta)
            assert np.allclose(Es, oE, rtol=0, atol=1e-9)
            d.close()

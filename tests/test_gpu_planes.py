"""Bit-plane uniforms (mcx_lattice_set_uniforms PLANES) on the device: bit for bit against
the oracle's restatement, on both layouts, with the same equilibrium as the per-site
words (GPU)."""
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _pair(mcx, L, beta, seed=42, stream=0, nsweeps=4, layout="int8", alg="metropolis", h=0.0, ctx=None):
    sys_ = mcx.Ising(L, h=h, layout=layout, ctx=ctx)
    sys_.set_uniforms("planes")
    mcx.init_(sys_, "random", rng=mcx.Philox(seed, stream))
    s = O.init_random(O.ISING, L, seed, stream)
    a = {"metropolis": mcx.Metropolis, "glauber": mcx.Glauber, "heatbath": mcx.HeatBath}[alg](
        mcx.Philox(seed, stream), beta=beta)
    obs = mcx.sweep_(sys_, a, nsweeps, record=True)
    oalg = {"metropolis": O.METROPOLIS, "glauber": O.GLAUBER, "heatbath": O.HEATBATH}[alg]
    oobs, att, acc = O.cb_sweep(s, O.ISING, L, oalg, beta, seed, stream=stream, nsweeps=nsweeps, h=h, uniforms=1)
    return sys_, a, obs, s, oobs, att, acc


CASES = [
    # dims, beta: 2-D and 3-D, one word per row and many, thresholds of 0 (beta 3) and
    # thresholds whose low 24 bits decide often (beta near 0)
    ([128, 128], 0.4407),
    ([256, 64], 0.3),
    ([1024, 96], 0.6),
    ([128, 128], 3.0),
    ([128, 64], 0.02),
    ([128, 16, 8], 0.2216),
    ([256, 12, 10], 0.5),
]


@pytest.mark.parametrize("layout", ["int8", "msc64"])
@pytest.mark.parametrize("L,beta", CASES)
def test_planes_parity(gpu, L, beta, layout):
    sys_, a, obs, s, oobs, att, acc = _pair(gpu, L, beta, seed=5, stream=1, layout=layout)
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert a.accepted == acc and a.steps == att
    sys_.close()


GLAUBER_CASES = [([128, 128], 0.4407), ([256, 64], 0.3), ([1024, 96], 0.6), ([128, 64], 0.0),
                 ([128, 16, 8], 0.2216), ([256, 12, 10], 3.0)]


@pytest.mark.parametrize("layout", ["int8", "msc64"])
@pytest.mark.parametrize("L,beta", GLAUBER_CASES)
def test_planes_glauber_parity(gpu, L, beta, layout):
    """Glauber without a field (the class form: a threshold for every aligned count) with
    bit-plane uniforms on the packed words, against the oracle; beta 0 (every threshold 2^31)
    and beta 3 (thresholds near 0 and near 2^32)."""
    sys_, a, obs, s, oobs, att, acc = _pair(gpu, L, beta, seed=9, stream=2, layout=layout, alg="glauber")
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert a.accepted == acc and a.steps == att
    sys_.close()


def test_planes_l4096_bit_exact(gpu):
    """2-D L=4096, seed 7, Metropolis at beta 0.4407: two sweeps of the plane form against
    the oracle, both layouts."""
    L = [4096, 4096]
    s = O.init_random(O.ISING, L, 7)
    oobs, _, acc = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.4407, 7, nsweeps=2, uniforms=1)
    for layout in ("int8", "msc64"):
        sys_ = gpu.Ising(L, layout=layout)
        sys_.set_uniforms("planes")
        gpu.init_(sys_, "random", rng=gpu.Philox(7))
        a = gpu.Metropolis(gpu.Philox(7), beta=0.4407)
        obs = gpu.sweep_(sys_, a, 2, record=True)
        assert np.array_equal(obs, oobs)
        assert a.accepted == acc
        assert np.array_equal(sys_.spins, s)
        sys_.close()
    # Glauber at the configured beta 0.30, int8 storage
    s = O.init_random(O.ISING, L, 7)
    oobs, _, acc = O.cb_sweep(s, O.ISING, L, O.GLAUBER, 0.3, 7, nsweeps=2, uniforms=1)
    sys_ = gpu.Ising(L)
    sys_.set_uniforms("planes")
    gpu.init_(sys_, "random", rng=gpu.Philox(7))
    a = gpu.Glauber(gpu.Philox(7), beta=0.3)
    obs = gpu.sweep_(sys_, a, 2, record=True)
    assert np.array_equal(obs, oobs) and a.accepted == acc and np.array_equal(sys_.spins, s)
    sys_.close()


GENERAL_CASES = [  # alg, h, dims, beta: heat bath and fields (the general form), always / never classes at beta 3
    ("heatbath", 0.0, [256, 64], 0.44), ("heatbath", 0.2, [128, 128], 0.3), ("heatbath", 0.0, [128, 16, 8], 0.2216),
    ("heatbath", -0.1, [256, 12, 10], 3.0), ("metropolis", 0.3, [256, 64], 0.44), ("metropolis", -0.5, [128, 16, 8], 3.0),
    ("glauber", 0.2, [1024, 96], 0.6), ("glauber", -0.2, [256, 12, 10], 0.25),
]


@pytest.mark.parametrize("layout", ["int8", "msc64"])
@pytest.mark.parametrize("alg,h,L,beta", GENERAL_CASES)
def test_planes_general_form_parity(gpu, alg, h, L, beta, layout):
    """Every other Ising rule (heat bath; Metropolis and Glauber with a field) with bit-plane
    uniforms on the packed words, against the oracle: flips, series and counters."""
    sys_, a, obs, s, oobs, att, acc = _pair(gpu, L, beta, seed=11, stream=3, layout=layout, alg=alg, h=h)
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert (a.flips if alg == "heatbath" else a.accepted) == acc
    sys_.close()


BC_CASES = [
    # dims, rule, beta, D, sweeps: one block (8^2, 32^2), a thread-block cluster (128 x 96), the
    # per-site kernel (W = 3), the strip kernel (2048^2, 3-D), captured sweep graphs (66 sweeps
    # of 1024 x 544), heat bath (no proposal: the per-site chain)
    ([8, 8], "metropolis", 0.5, 1.0, 4), ([32, 32], "glauber", 0.6, 0.5, 4), ([128, 96], "metropolis", 0.6, 1.0, 4),
    ([6, 8], "metropolis", 0.5, 0.7, 4), ([2048, 2048], "metropolis", 0.6, 1.0, 2), ([32, 16, 8], "glauber", 0.35, 0.7, 4),
    ([1024, 544], "metropolis", 0.6, 1.0, 66), ([2048, 1024], "heatbath", 0.6, 1.0, 3),
]


@pytest.mark.parametrize("L,alg,beta,D,nsweeps", BC_CASES)
def test_bc_planes_parity(gpu, L, alg, beta, D, nsweeps):
    """Blume-Capel with bit-plane proposal bits on every launch form, against the oracle."""
    sys_ = gpu.BlumeCapel(L, D=D)
    sys_.set_uniforms("planes")
    gpu.init_(sys_, "random", rng=gpu.Philox(13, 1))
    a = {"metropolis": gpu.Metropolis, "glauber": gpu.Glauber, "heatbath": gpu.HeatBath}[alg](gpu.Philox(13, 1),
                                                                                            beta=beta)
    obs = gpu.sweep_(sys_, a, nsweeps, record=True)
    s = O.init_random(O.BC, L, 13, 1)
    oalg = {"metropolis": O.METROPOLIS, "glauber": O.GLAUBER, "heatbath": O.HEATBATH}[alg]
    oobs, att, acc = O.cb_sweep(s, O.BC, L, oalg, beta, 13, stream=1, nsweeps=nsweeps, D=D, uniforms=1)
    assert np.array_equal(obs, oobs)
    assert np.array_equal(sys_.spins, s)
    assert (a.flips if alg == "heatbath" else a.accepted) == acc
    sys_.close()


def test_bc_planes_batch(gpu):
    """Independent Blume-Capel chains with bit planes in one mcx_sweep_batch call (the one-block
    batch form) against their oracle runs; a per-site lattice in the same batch keeps its words."""
    systems, algs = [], []
    for i, u in enumerate(("planes", "site", "planes")):
        b = gpu.BlumeCapel([32, 32], D=0.6)
        b.set_uniforms(u)
        gpu.init_(b, "random", rng=gpu.Philox(40 + i, i))
        systems.append(b)
        algs.append(gpu.Metropolis(gpu.Philox(50 + i, i), beta=0.5 + 0.05 * i))
    obs = gpu.sweep_batch_(systems, algs, 7, record=True)
    for i, u in enumerate(("planes", "site", "planes")):
        s = O.init_random(O.BC, [32, 32], 40 + i, i)
        oo, _, acc = O.cb_sweep(s, O.BC, [32, 32], O.METROPOLIS, 0.5 + 0.05 * i, 50 + i, stream=i, nsweeps=7, D=0.6,
                                uniforms=1 if u == "planes" else 0)
        assert np.array_equal(obs[i], oo) and np.array_equal(systems[i].spins, s) and algs[i].accepted == acc
        systems[i].close()


def test_planes_calls_compose_and_switch(gpu):
    """3 + 5 sweeps equal 8; switching back to per-site words continues the same lattice
    with the per-site stream; a heat-bath call in between (the general form) continues it."""
    L = [512, 256]
    sys_ = gpu.Ising(L)
    sys_.set_uniforms("planes")
    gpu.init_(sys_, "random", rng=gpu.Philox(3))
    a = gpu.Metropolis(gpu.Philox(3), beta=0.45)
    o1 = gpu.sweep_(sys_, a, 3, record=True)
    o2 = gpu.sweep_(sys_, a, 5, record=True)
    s = O.init_random(O.ISING, L, 3)
    oo, _, acc = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.45, 3, nsweeps=8, uniforms=1)
    assert np.array_equal(np.concatenate([o1, o2]), oo) and np.array_equal(sys_.spins, s)
    hb = gpu.HeatBath(gpu.Philox(4), beta=0.45)
    gpu.sweep_(sys_, hb, 2)
    O.cb_sweep(s, O.ISING, L, O.HEATBATH, 0.45, 4, nsweeps=2, uniforms=1)
    assert np.array_equal(sys_.spins, s)
    sys_.set_uniforms("site")
    o3 = gpu.sweep_(sys_, a, 4, record=True)
    oo3, _, _ = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.45, 3, sweep0=8, nsweeps=4)
    assert np.array_equal(o3, oo3) and np.array_equal(sys_.spins, s)
    sys_.close()


def test_planes_batch_and_checkpoint(gpu, tmp_path):
    """mcx_sweep_batch runs plane lattices one mcx_sweep each (same results); a checkpoint
    keeps the form."""
    from mcx import checkpoint as K
    dims = [[128, 128], [256, 128]]
    systems, algs = [], []
    for i, L in enumerate(dims):
        sysd = gpu.Ising(L)
        sysd.set_uniforms("planes")
        gpu.init_(sysd, "random", rng=gpu.Philox(10 + i, i))
        systems.append(sysd)
        algs.append(gpu.Metropolis(gpu.Philox(20 + i, i), beta=0.4 + 0.05 * i))
    obs = gpu.sweep_batch_(systems, algs, 6, record=True)
    for i, L in enumerate(dims):
        s = O.init_random(O.ISING, L, 10 + i, i)
        oo, _, acc = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.4 + 0.05 * i, 20 + i, stream=i, nsweeps=6, uniforms=1)
        assert np.array_equal(obs[i], oo) and np.array_equal(systems[i].spins, s) and algs[i].accepted == acc
    f = str(tmp_path / "planes.ckpt")
    ck = K.init_checkpoint(f, sys=systems[1], alg=algs[1], sweep=6)
    a = gpu.sweep_(systems[1], algs[1], 5, record=True)
    r = K.restore_checkpoint(f)
    assert r.sys.uniforms == "planes"
    b = gpu.sweep_(r.sys, r.alg, 5, record=True)
    assert np.array_equal(a, b) and np.array_equal(systems[1].spins, r.sys.spins)
    K.finalize_(ck)


def test_planes_argument_errors(gpu):
    for L in ([64, 64], [96, 32], [200, 8]):
        s = gpu.Ising(L)
        with pytest.raises(gpu.ArgumentError):
            s.set_uniforms("planes")
        s.close()
    # the int8 kernels draw per-site words: packing off leaves no way to run the plane form
    s = gpu.Ising([128, 64])
    s.set_uniforms("planes")
    s.set_packing(False)
    for kind in (gpu.Metropolis, gpu.HeatBath):
        with pytest.raises(gpu.ArgumentError):
            gpu.sweep_(s, kind(gpu.Philox(1), beta=0.4), 1)
    s.set_uniforms("site")
    gpu.sweep_(s, gpu.HeatBath(gpu.Philox(1), beta=0.4), 1)  # per-site words: fine
    s.close()


def test_planes_budget(gpu):
    """The plane form of an int8 lattice needs its packed copy: with no room in the budget
    the call fails with BudgetError and leaves the lattice and the stream untouched."""
    L = [1024, 512]
    probe = gpu.Context()
    lat = gpu.Ising(L, ctx=probe)
    used = probe.memory()[0]
    lat.close()
    probe.close()
    ctx = gpu.Context(hbm_budget=used + (4 << 10))
    s = gpu.Ising(L, ctx=ctx)
    s.set_uniforms("planes")
    gpu.init_(s, "random", rng=gpu.Philox(2))
    before = s.spins
    a = gpu.Metropolis(gpu.Philox(2), beta=0.4)
    with pytest.raises(gpu.BudgetError):
        gpu.sweep_(s, a, 4)
    assert np.array_equal(s.spins, before) and a.rng.counter == 0
    s.close()


def test_planes_refused_by_noalloc(gpu):
    import ctypes as C
    lib = gpu._lib.load()
    fn = lib.mcx_sweep_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(gpu._lib.mcx_rng), C.c_int64, C.c_void_p,
                   C.c_void_p]
    s = gpu.Ising([128, 64])
    s.set_uniforms("planes")
    r = gpu._lib.mcx_rng(1, 0, 0, 0)
    assert fn(s.handle, 0, 0.4, C.byref(r), 2, None, None) == 1  # MCX_ERR_INVALID_ARG
    assert fn(s.handle, 2, 0.4, C.byref(r), 2, None, None) == 1  # heat bath draws planes too
    s.set_uniforms("site")
    assert fn(s.handle, 2, 0.4, C.byref(r), 2, None, None) == 0
    s.close()


@pytest.mark.parametrize("alg,beta,start", [("metropolis", 0.4407, "random"), ("glauber", 0.3, "random"),
                                             ("glauber", 0.6, "up"), ("heatbath", 0.3, "random"),
                                             ("heatbath", 0.6, "up")])
def test_planes_kaufman_l128(gpu, alg, beta, start):
    """16 independent 128^2 chains with plane uniforms (10^3 thermalisation + 5000 recorded
    sweeps): the mean energy per site within 3 standard errors of the chain means of
    Kaufman's exact finite-torus value.  Metropolis at beta 0.4407; Glauber and heat bath
    (the same flip probabilities, slower to relax) off beta_c: at 0.4407 both the per-site and
    the plane form of the oracle's heat bath sit at -1.398 after these sweeps from a random
    start, against the exact -1.4192."""
    from mcx.analysis import kaufman_ising2d
    L, nch = 128, 16
    means = []
    for i in range(nch):
        c = gpu.Ising([L, L])
        c.set_uniforms("planes")
        if start == "random":
            gpu.init_(c, "random", rng=gpu.Philox(42, i))
        else:
            gpu.init_(c, start)
        a = {"metropolis": gpu.Metropolis, "glauber": gpu.Glauber, "heatbath": gpu.HeatBath}[alg](gpu.Philox(42, i),
                                                                                                beta=beta)
        gpu.sweep_(c, a, 1000)
        obs = gpu.sweep_(c, a, 5000, record=True)
        means.append((-obs[:, 0] / (L * L)).mean())
        c.close()
    means = np.array(means)
    exact = kaufman_ising2d(L, L, beta)[1] / (L * L)
    se = means.std(ddof=1) / math.sqrt(nch)
    assert abs(means.mean() - exact) < 3 * se, (means.mean(), exact, se)


@pytest.mark.parametrize("alg", ["metropolis", "glauber", "heatbath"])
def test_planes_antiferromagnet(gpu, alg):
    """J = -1: the thresholds fit neither the rank nor the class form (some classes always
    flip), so every rule takes the general form; against the oracle on both layouts."""
    L = [256, 32]
    for layout in ("int8", "msc64"):
        sys_ = gpu.Ising(L, J=-1.0, layout=layout)
        sys_.set_uniforms("planes")
        gpu.init_(sys_, "random", rng=gpu.Philox(17))
        a = {"metropolis": gpu.Metropolis, "glauber": gpu.Glauber, "heatbath": gpu.HeatBath}[alg](gpu.Philox(17),
                                                                                                beta=0.5)
        obs = gpu.sweep_(sys_, a, 3, record=True)
        s = O.init_random(O.ISING, L, 17)
        oalg = {"metropolis": O.METROPOLIS, "glauber": O.GLAUBER, "heatbath": O.HEATBATH}[alg]
        oobs, _, acc = O.cb_sweep(s, O.ISING, L, oalg, 0.5, 17, nsweeps=3, J=-1.0, uniforms=1)
        assert np.array_equal(obs, oobs) and np.array_equal(sys_.spins, s)
        assert (a.flips if alg == "heatbath" else a.accepted) == acc
        sys_.close()


def test_bc_planes_noalloc(gpu):
    """mcx_sweep_noalloc on a Blume-Capel lattice with bit-plane proposals equals mcx_sweep on a
    twin lattice, bit for bit, over two calls."""
    import ctypes as C
    import torch
    lib = gpu._lib.load()
    fn = lib.mcx_sweep_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(gpu._lib.mcx_rng), C.c_int64, C.c_void_p,
                   C.c_void_p]
    a = gpu.BlumeCapel([256, 64], D=0.8)
    b = gpu.BlumeCapel([256, 64], D=0.8)
    for x in (a, b):
        x.set_uniforms("planes")
        gpu.init_(x, "random", rng=gpu.Philox(21))
    ra = gpu._lib.mcx_rng(5, 0, 2, 0)
    rb = gpu._lib.mcx_rng(5, 0, 2, 0)
    for n in (5, 9):
        oa = np.zeros((n, 3), np.int64)
        gpu._check(lib.mcx_sweep(a.handle, 0, 0.6, C.byref(ra), n, oa.ctypes.data, None))
        ob = torch.full((n, 3), -1, dtype=torch.int64, device="cuda")
        gpu._check(fn(b.handle, 0, 0.6, C.byref(rb), n, ob.data_ptr(), None))
        torch.cuda.synchronize()
        assert np.array_equal(oa, ob.cpu().numpy()) and np.array_equal(a.spins, b.spins)
    a.close()
    b.close()

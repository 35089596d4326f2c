"""The oracle's bit-plane uniforms (CPU): the definition against raw Philox blocks, the
rules it applies to, and the same equilibrium as the per-site words."""
import numpy as np
import pytest

import oracle as O

P_PLANES, P_TAIL = 9, 10


def _block(seed, stream, sweep, colour, purpose, x):
    w2 = ((sweep >> 32) & 0xFFFF) | (colour << 16) | (purpose << 24)
    return [int(v) for v in O.philox([x & 0xFFFFFFFF, sweep & 0xFFFFFFFF, w2, stream],
                                     [seed & 0xFFFFFFFF, seed >> 32])]


def _plane_uniform(seed, stream, sweep, colour, e):
    b, u = e & 63, 0
    for j in range(4):
        o = _block(seed, stream, sweep, colour, P_PLANES, (e >> 6) * 16 + j)
        p0, p1 = o[0] | (o[1] << 32), o[2] | (o[3] << 32)
        u |= ((p0 >> b) & 1) << (31 - 2 * j)
        u |= ((p1 >> b) & 1) << (30 - 2 * j)
    return u | (_block(seed, stream, sweep, colour, P_TAIL, e >> 2)[e & 3] & 0xFFFFFF)


def test_plane_uniform_definition():
    for seed, stream, sweep in ((7, 0, 0), (2 ** 40 + 3, 5, 2 ** 33 + 9), (123, 1, 77)):
        for colour in (0, 1):
            for e in (0, 1, 3, 4, 63, 64, 65, 127, 1000, 2 ** 20 + 17):
                assert O.plane_uniform(seed, stream, sweep, colour, e) == _plane_uniform(seed, stream, sweep,
                                                                                          colour, e)


def test_plane_uniform_bits_are_balanced():
    us = np.array([O.plane_uniform(11, 0, 3, 1, e) for e in range(1 << 14)], np.uint64)
    for bit in (31, 28, 24, 23, 12, 0):  # plane bits and tail bits
        frac = float(((us >> np.uint64(bit)) & np.uint64(1)).mean())
        assert abs(frac - 0.5) < 4 * 0.5 / np.sqrt(us.size), (bit, frac)
    # the top byte (the planes) is uniform over its 256 values
    counts = np.bincount((us >> np.uint64(24)).astype(np.int64), minlength=256)
    exp = us.size / 256
    assert ((counts - exp) ** 2 / exp).sum() < 255 + 6 * np.sqrt(2 * 255)


def test_plane_uniforms_of_neighbouring_sites_are_uncorrelated():
    """Sites e and e + 1 (and e + 64, the same bit of the next plane word) take their top bits
    from neighbouring bits of the same Philox words: their correlation is within 4 sigma of 0."""
    us = np.array([O.plane_uniform(13, 2, 9, 0, e) for e in range(1 << 14)], np.float64)
    x = (us - us.mean()) / us.std()
    for lag in (1, 2, 64):
        r = float((x[:-lag] * x[lag:]).mean())
        assert abs(r) < 4 / np.sqrt(x.size - lag), (lag, r)


@pytest.mark.parametrize("alg,h", [(O.METROPOLIS, 0.0), (O.GLAUBER, 0.0), (O.HEATBATH, 0.0), (O.METROPOLIS, 0.2),
                                   (O.GLAUBER, -0.2), (O.HEATBATH, 0.3)])
def test_planes_change_the_chain(alg, h):
    """Every Ising rule draws bit planes once asked (the per-site chain differs)."""
    L = [128, 8]
    a = O.init_random(O.ISING, L, 5)
    b = a.copy()
    O.cb_sweep(a, O.ISING, L, alg, 0.44, 5, nsweeps=2, h=h)
    O.cb_sweep(b, O.ISING, L, alg, 0.44, 5, nsweeps=2, h=h, uniforms=1)
    assert not np.array_equal(a, b)


@pytest.mark.parametrize("L", [[64, 64], [96, 8]])
def test_planes_need_an_ising_lattice_with_lx_multiple_of_128(L):
    s = O.init_random(O.ISING, L, 1)
    with pytest.raises(ValueError):
        O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.4, 1, nsweeps=1, uniforms=1)


def test_bc_plane_bit_definition():
    """Blume-Capel proposal bit e: bit e & 63 of plane e >> 6, planes 2m, 2m+1 = words
    0 | 1 << 32 and 2 | 3 << 32 of the block at counter m."""
    for seed, stream, sweep in ((7, 0, 0), (2 ** 40 + 3, 5, 2 ** 33 + 9)):
        for colour in (0, 1):
            for e in (0, 1, 31, 32, 63, 64, 100, 127, 128, 1000, 2 ** 20 + 77):
                o = _block(seed, stream, sweep, colour, P_PLANES, e >> 7)
                plane = (o[2] | (o[3] << 32)) if (e >> 6) & 1 else (o[0] | (o[1] << 32))
                assert O.bc_plane_bit(seed, stream, sweep, colour, e) == (plane >> (e & 63)) & 1


@pytest.mark.parametrize("alg,changes", [(O.METROPOLIS, True), (O.GLAUBER, True), (O.HEATBATH, False)])
def test_bc_planes_replace_the_proposal_bits(alg, changes):
    """On a Blume-Capel lattice (any size) bit planes replace the proposal words; heat bath
    has no proposal and keeps its chain."""
    L = [10, 6]
    a = O.init_random(O.BC, L, 5)
    b = a.copy()
    oa = O.cb_sweep(a, O.BC, L, alg, 0.5, 5, nsweeps=3, D=0.7)
    ob = O.cb_sweep(b, O.BC, L, alg, 0.5, 5, nsweeps=3, D=0.7, uniforms=1)
    assert (not np.array_equal(a, b)) == changes
    if not changes:
        assert np.array_equal(oa[0], ob[0])


@pytest.mark.parametrize("alg", [O.METROPOLIS, O.GLAUBER])
def test_bc_planes_sample_the_same_equilibrium(alg):
    """Blume-Capel 64 x 64, D = 1, beta = 0.4 (disordered): <E>/N and <Q>/N (the density of
    non-zero spins) of the two forms agree within 4 combined sigma of 20-sweep bins."""
    L = [64, 64]
    res = []
    for u in (0, 1):
        s = O.init_random(O.BC, L, 31 + u)
        O.cb_sweep(s, O.BC, L, alg, 0.4, 31 + u, nsweeps=200, D=1.0, record=False, uniforms=u)
        obs, _, _ = O.cb_sweep(s, O.BC, L, alg, 0.4, 31 + u, sweep0=200, nsweeps=1200, D=1.0, uniforms=u)
        e = (-obs[:, 0] + 1.0 * obs[:, 2]) / s.size  # E = -J sum s_i s_j + D sum s_i^2
        q = obs[:, 2] / s.size
        res.append([(x.reshape(60, 20).mean(axis=1).mean(), x.reshape(60, 20).mean(axis=1).std(ddof=1) / np.sqrt(60))
                     for x in (e, q)])
    for k in range(2):
        (m0, s0), (m1, s1) = res[0][k], res[1][k]
        assert abs(m0 - m1) < 4 * np.hypot(s0, s1), (k, m0, m1, s0, s1)


def _energy_series(uniforms, beta, L, nsweeps, burn, seed, alg=O.METROPOLIS):
    s = O.init_random(O.ISING, L, seed)
    O.cb_sweep(s, O.ISING, L, alg, beta, seed, nsweeps=burn, record=False, uniforms=uniforms)
    obs, _, _ = O.cb_sweep(s, O.ISING, L, alg, beta, seed, sweep0=burn, nsweeps=nsweeps, uniforms=uniforms)
    return -obs[:, 0].astype(float) / s.size


@pytest.mark.parametrize("beta,alg", [(0.3, O.METROPOLIS), (0.6, O.METROPOLIS), (0.3, O.GLAUBER), (0.3, O.HEATBATH)])
def test_planes_sample_the_same_equilibrium(beta, alg):
    """<E>/N of the two forms (128 x 128, 600 sweeps after 100) agree within 4 combined
    sigma of 20-sweep bins, and both sit on Onsager's infinite-lattice energy (finite-size
    corrections are exponentially small away from beta_c).  Glauber runs at 0.3: from a
    random start its domains at 0.6 do not coarsen within the 100 sweeps."""
    L = [128, 128]
    means, errs = [], []
    for u in (0, 1):
        e = _energy_series(u, beta, L, 600, 100, 21 + u, alg)
        bins = e.reshape(30, 20).mean(axis=1)
        means.append(bins.mean())
        errs.append(bins.std(ddof=1) / np.sqrt(bins.size))
    assert abs(means[0] - means[1]) < 4 * np.hypot(*errs), (means, errs)
    from scipy.special import ellipk
    k = 2 * np.sinh(2 * beta) / np.cosh(2 * beta) ** 2
    exact = -1 / np.tanh(2 * beta) * (1 + 2 / np.pi * (2 * np.tanh(2 * beta) ** 2 - 1) * ellipk(k * k))
    for m, s in zip(means, errs):
        assert abs(m - exact) < 4 * s + 1e-4, (m, exact, s)

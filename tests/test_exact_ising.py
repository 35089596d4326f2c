"""Kaufman's exact finite-torus 2-D Ising results (mcx.analysis.kaufman_ising2d) against the
exact 8x8 density of states the reference ships (SpinSystems/data/exact_solutions/
ising2D_8x8.csv, read by SpinSystems/src/ising2d_exact.jl:1-42), brute-force enumeration of
small tori, Onsager's infinite-lattice energy and finite differences (CPU)."""
import json
import math
import os

import numpy as np
import pytest

from mcx.analysis import kaufman_ising2d, onsager_energy_per_site


def _dos8():
    d = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ising2d_8x8_logdos.json")))
    return (np.array([e for e, _ in d["energy_logdos"]], float), np.array([v for _, v in d["energy_logdos"]]))


@pytest.mark.parametrize("beta", [0.1, 0.3, 0.4, 0.4407, 0.5, 1.0])
def test_l8_against_exact_density_of_states(beta):
    E, lg = _dos8()
    lw = lg - beta * E
    mx = lw.max()
    w = np.exp(lw - mx)
    lz = mx + math.log(w.sum())
    e = float((w * E).sum() / w.sum())
    klz, ke = kaufman_ising2d(8, 8, beta)
    assert abs(klz - lz) <= 1e-12 * abs(lz)
    assert abs(ke - e) <= 1e-10 * 128


def _enumerate(m, n, beta):
    N = m * n
    c = np.arange(1 << N, dtype=np.int64)
    s = np.array([((c >> i) & 1) * 2 - 1 for i in range(N)], dtype=np.int8)
    E = np.zeros(1 << N)
    for y in range(m):
        for x in range(n):
            i, j, k = y * n + x, y * n + (x + 1) % n, ((y + 1) % m) * n + x
            E -= s[i].astype(float) * s[j] + s[i].astype(float) * s[k]
    lw = -beta * E
    mx = lw.max()
    w = np.exp(lw - mx)
    return mx + math.log(w.sum()), float((w * E).sum() / w.sum())


@pytest.mark.parametrize("m,n", [(4, 4), (3, 4), (5, 4), (3, 5)])
@pytest.mark.parametrize("beta", [0.2, 0.37, 0.8])
def test_small_tori_against_enumeration(m, n, beta):
    lz, e = _enumerate(m, n, beta)
    klz, ke = kaufman_ising2d(m, n, beta)
    assert abs(klz - lz) <= 1e-12 * abs(lz) and abs(ke - e) <= 1e-10 * 2 * m * n


@pytest.mark.parametrize("beta", [0.3, 0.6])
def test_large_torus_approaches_onsager(beta):
    L = 4096
    assert abs(kaufman_ising2d(L, L, beta)[1] / (L * L) - onsager_energy_per_site(beta)) < 1e-12


@pytest.mark.parametrize("L,beta", [(64, 0.4407), (256, 0.43), (16, 0.6)])
def test_energy_is_the_derivative_of_log_z(L, beta):
    h = 1e-6
    d = (kaufman_ising2d(L, L, beta + h)[0] - kaufman_ising2d(L, L, beta - h)[0]) / (2 * h)
    e = kaufman_ising2d(L, L, beta)[1]
    assert abs(-d - e) <= 1e-6 * abs(e)

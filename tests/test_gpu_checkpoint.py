"""Checkpoint / resume of device state (GPU): a restored run continues bit for bit
(test/test_checkpointing.jl:100-147 restated for the device objects)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_lattice_and_algorithm_resume(gpu, tmp_path):
    from mcx import checkpoint as K
    sys_ = gpu.Ising([64, 32])
    gpu.init_(sys_, "random", rng=gpu.Philox(8))
    alg = gpu.Metropolis(gpu.Philox(8), beta=0.45)
    gpu.sweep_(sys_, alg, 10)
    f = str(tmp_path / "run.ckpt")
    ck = K.init_checkpoint(f, sys=sys_, alg=alg, sweep=10)
    a = gpu.sweep_(sys_, alg, 15, record=True)
    r = K.restore_checkpoint(f)
    assert r.sweep == 10
    b = gpu.sweep_(r.sys, r.alg, 15, record=True)
    assert np.array_equal(a, b) and np.array_equal(sys_.spins, r.sys.spins)
    assert (alg.steps, alg.accepted) == (r.alg.steps, r.alg.accepted)
    K.finalize_(ck)
    assert not os.path.exists(f)


def test_parallel_tempering_resume(gpu, tmp_path):
    from mcx import checkpoint as K
    from mcx.pt import ParallelTempering
    lad = [(16, [0.25, 0.23, 0.21]), (8, [0.3, 0.25, 0.2])]
    pt = ParallelTempering(lad, dim=3, seed=3)
    pt.init_(3)
    pt.sweep_(5)
    f = str(tmp_path / "pt.ckpt")
    K.init_checkpoint(f, pt=pt)
    pt.sweep_(6, mode="plain")
    r = K.restore_checkpoint(f).pt
    r.sweep_(6)
    assert np.array_equal(pt.positions, r.positions) and pt.stage == r.stage
    assert all(np.array_equal(x, y) for x, y in zip(pt.counters(), r.counters()))
    for k in range(pt.nrep):
        assert np.array_equal(pt.spins(k), r.spins(k))


def test_wang_landau_resume(gpu, tmp_path):
    from mcx import checkpoint as K
    from mcx import flathist as F
    s = gpu.BlumeCapel([16, 16], D=1.0)
    gpu.init_(s, "random", rng=gpu.Philox(5))
    alg = F.WangLandau(gpu.Philox(5), F.WangLandauEnsemble((-256, 1, 1025), logf=0.5))
    F.sweep_walkers_([s], [alg], 7)
    F.flatness(alg.ensemble)  # sets visited marks
    f = str(tmp_path / "wl.ckpt")
    K.init_checkpoint(f, s=s, alg=alg)
    F.sweep_walkers_([s], [alg], 9)
    r = K.restore_checkpoint(f)
    F.sweep_walkers_([r.s], [r.alg], 9)
    assert np.array_equal(s.spins, r.s.spins)
    assert np.array_equal(alg.ensemble.logweight, r.alg.ensemble.logweight)
    assert np.array_equal(alg.ensemble.histogram, r.alg.ensemble.histogram)
    assert F.flatness(alg.ensemble) == F.flatness(r.alg.ensemble)
    assert (alg.steps, alg.accepted) == (r.alg.steps, r.alg.accepted)


def test_graph_resume(gpu, tmp_path):
    """An IsingMatrix spin glass with a field per site: the restored run repeats the spins
    and counters bit for bit; energies agree to FP64 summation order."""
    from mcx import checkpoint as K
    from mcx.graph import IsingGraphDevice
    from graph_cases import from_edges, random_edges
    es = random_edges(500, 1200, 12)
    rp, col, val = from_edges(500, es, np.random.default_rng(13).normal(size=len(es)))
    s = IsingGraphDevice(rp, col, val, h=np.random.default_rng(14).normal(size=500) * 0.2)
    gpu.init_(s, "random", rng=gpu.Philox(4))
    alg = gpu.Glauber(gpu.Philox(4), beta=0.9)
    gpu.sweep_(s, alg, 5)
    f = str(tmp_path / "graph.ckpt")
    K.init_checkpoint(f, s=s, alg=alg)
    Ea, Ma = gpu.sweep_(s, alg, 8, record=True)
    r = K.restore_checkpoint(f)
    Eb, Mb = gpu.sweep_(r.s, r.alg, 8, record=True)
    assert np.array_equal(s.spins, r.s.spins) and np.array_equal(Ma, Mb)
    assert np.allclose(Ea, Eb, rtol=0, atol=1e-9)
    assert (alg.steps, alg.accepted) == (r.alg.steps, r.alg.accepted)

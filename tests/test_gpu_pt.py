"""Batched parallel tempering on the device against the oracle (GPU)."""
import numpy as np
import pytest

import oracle as O
from oracle_runs import oracle_pt

pytestmark = pytest.mark.gpu

CASES = [
    (3, [(8, [0.25, 0.235, 0.22]), (16, [0.25, 0.24, 0.23, 0.2])], "metropolis", 7, 1),
    (3, [(24, [0.23, 0.22, 0.21]), (48, [0.22, 0.2])], "glauber", 5, 1),
    (2, [(16, [0.6, 0.5, 0.45, 0.4, 0.3]), (32, [0.5, 0.44])], "heatbath", 8, 2),
    (2, [(64, [0.45, 0.44, 0.43, 0.42]), (8, [0.9, 0.1])], "metropolis", 9, 1),
]


@pytest.mark.parametrize("mode", ["persistent", "plain"])
@pytest.mark.parametrize("dim,ladders,alg,nsweeps,every", CASES)
def test_pt_parity(gpu, mode, dim, ladders, alg, nsweeps, every):
    from mcx.pt import ParallelTempering
    seed = 123
    pt = ParallelTempering(ladders, dim=dim, seed=seed)
    pt.init_(seed)
    series = pt.sweep_(nsweeps, alg=alg, exchange_every=every, mode=mode, record=True)
    spins, oseries, opos, ostage, osteps, oacc = oracle_pt(ladders, dim, alg, seed, nsweeps, every)
    assert np.array_equal(series, oseries)
    assert np.array_equal(pt.positions, opos)
    assert pt.stage == ostage
    s, a = pt.counters()
    assert np.array_equal(s, osteps) and np.array_equal(a, oacc)
    for r in range(pt.nrep):
        assert np.array_equal(pt.spins(r), spins[r]), r
    P, M = pt.observables()
    assert np.array_equal(P, oseries[-1, :, 0]) and np.array_equal(M, oseries[-1, :, 1])


def test_pt_runs_compose(gpu):
    """3 + 4 sweeps in two calls equal 7 sweeps in one (stage and counters carry over)."""
    from mcx.pt import ParallelTempering
    lad = [(16, [0.25, 0.23, 0.21]), (8, [0.3, 0.2])]
    a = ParallelTempering(lad, dim=3, seed=5)
    a.init_(5)
    a.sweep_(3)
    a.sweep_(4, mode="plain")
    b = ParallelTempering(lad, dim=3, seed=5)
    b.init_(5)
    b.sweep_(7)
    assert np.array_equal(a.positions, b.positions) and a.stage == b.stage
    assert np.array_equal(a.counters()[1], b.counters()[1])
    for r in range(a.nrep):
        assert np.array_equal(a.spins(r), b.spins(r))


@pytest.mark.parametrize("alg,every", [("metropolis", 1), ("heatbath", 3)])
def test_distributed_ladder_matches_device_pt(gpu, alg, every):
    """Ladder 1 of a two-ladder ParallelTempering rerun by DistributedLadder in one process
    (device lattices swept by sweep_batch_, the exchange stage on the host through
    mcx_ladder_exchange): series, positions, stage, counters and spins are the kernel's."""
    from mcx.parallel import DistributedLadder
    from mcx.pt import ParallelTempering
    seed, n = 41, 11
    lad = [(8, [0.3, 0.25]), (16, [0.26, 0.25, 0.24, 0.235, 0.23, 0.22])]
    pt = ParallelTempering(lad, dim=3, seed=seed)
    pt.init_(seed)
    series = pt.sweep_(n, alg=alg, exchange_every=every, record=True)
    dl = DistributedLadder(16, lad[1][1], dim=3, seed=seed, ladder=1, stream0=2)
    dl.init_(seed)
    ds = np.concatenate([dl.sweep_(4, alg=alg, exchange_every=every, record=True),
                         dl.sweep_(n - 4, alg=alg, exchange_every=every, record=True)])
    assert np.array_equal(ds, series[:, 2:])
    assert np.array_equal(dl.positions, pt.positions[2:])
    assert dl.stage == pt.stage
    s, a = pt.counters()
    assert np.array_equal(dl.steps, s[1:]) and np.array_equal(dl.accepted, a[1:])
    for r in range(6):
        assert np.array_equal(dl.spins(r), pt.spins(2 + r)), r
    dl.close()


def test_bounded_wait_reports_timeout(gpu):
    """A device wait on a flag nothing sets gives up and reports, context intact."""
    ctx = gpu.default_context()
    with pytest.raises(gpu.DeviceTimeoutError):
        gpu._check(gpu._lib.load().mcx_wait_flag_test(ctx.handle, 1000))
    sys_ = gpu.Ising([8, 8])
    assert gpu.energy(sys_) == -128

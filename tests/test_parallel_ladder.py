"""One parallel-tempering ladder spread over processes (gloo on CPU, the oracle sweeping
each rank's replicas): the host exchange stage equals the oracle's, every rank reaches the
same positions, and the run does not depend on the number of ranks
(src/algorithms/replica_exchange.jl:227-243, the MPI form, restated over torch.distributed)."""
import os
import socket

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ALG = {"metropolis": O.METROPOLIS, "glauber": O.GLAUBER, "heatbath": O.HEATBATH}


class OracleSweeper:
    """Test stand-in for a rank's device: the oracle's checkerboard sweeps of replicas
    r0 .. r1-1, replica r on stream stream0 + r."""

    def __init__(self, L, dim, r0, r1, stream0=0):
        self.dims, self.r0, self.s0 = [L] * dim, r0, r0 + stream0
        self.s = [None] * (r1 - r0)

    def init(self, seed):
        self.s = [O.init_random(O.ISING, self.dims, seed, self.s0 + i) for i in range(len(self.s))]

    def spins(self, i):
        return self.s[i].copy()

    def set_spins(self, i, values):
        self.s[i] = np.array(values, np.int8)

    def observables(self):
        return np.array([O.observables(s, self.dims)[:2] for s in self.s], np.int64).reshape(-1, 2)

    def sweep(self, betas, seed, t0, nsweeps, alg):
        out = np.zeros((nsweeps, len(self.s), 2), np.int64)
        for i, (s, b) in enumerate(zip(self.s, betas)):
            obs, _, _ = O.cb_sweep(s, O.ISING, self.dims, ALG[alg], float(b), seed, stream=self.s0 + i, sweep0=t0,
                                   nsweeps=nsweeps)
            out[:, i] = obs[:, :2]
        return out

    def close(self):
        pass


def oracle_ladder(L, dim, betas, seed, nsweeps, every, alg, ladder=0, J=1.0, h=0.0):
    """The single-process loop: sweep every replica once, exchange after every `every`-th."""
    n = len(betas)
    spins = [O.init_random(O.ISING, [L] * dim, seed, r) for r in range(n)]
    pos = np.arange(n, dtype=np.int32)
    steps = np.zeros(n - 1, np.uint64)
    acc = np.zeros(n - 1, np.uint64)
    stage = 0
    series = np.zeros((nsweeps, n, 2), np.int64)
    for t in range(nsweeps):
        for r in range(n):
            O.cb_sweep(spins[r], O.ISING, [L] * dim, ALG[alg], betas[pos[r]], seed, stream=r, sweep0=t, nsweeps=1,
                       J=J, h=h, record=False)
            series[t, r] = O.observables(spins[r], [L] * dim)[:2]
        if (t + 1) % every == 0:
            x = (-(J * series[t, :, 0].astype(np.float64))) - (h * series[t, :, 1].astype(np.float64))
            stage = O.pt_exchange(np.asarray(betas, np.float64), pos, stage, x, seed, ladder, t, steps, acc)
    return spins, series, pos, stage, steps, acc


CASE = dict(L=4, dim=3, betas=[0.30, 0.27, 0.245, 0.22, 0.2], seed=77, nsweeps=9, every=2, alg="metropolis")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run(P, c, backend, out_dir=None):
    rank = backend.rank if backend is not None else 0
    lad = P.DistributedLadder(c["L"], c["betas"], dim=c["dim"], seed=c["seed"], backend=backend,
                              sweeper=OracleSweeper(c["L"], c["dim"], *_bounds(len(c["betas"]), backend)))
    lad.init_(c["seed"])
    s1 = lad.sweep_(4, alg=c["alg"], exchange_every=c["every"], record=True)  # two calls compose
    s2 = lad.sweep_(c["nsweeps"] - 4, alg=c["alg"], exchange_every=c["every"], record=True)
    res = {"series": np.concatenate([s1, s2]), "pos": lad.positions, "stage": np.array([lad.stage]),
           "steps": lad.steps, "acc": lad.accepted, "obs": lad.observables(),
           "spins": np.concatenate([lad.spins(r) for r in lad.local_replicas()] + [np.zeros(0, np.int8)])}
    if out_dir is not None:
        for k, v in res.items():
            np.save(os.path.join(out_dir, "%s%d.npy" % (k, rank)), v)
    return res


def _bounds(n, backend):
    rank, size = (backend.rank, backend.size) if backend is not None else (0, 1)
    return n * rank // size, n * (rank + 1) // size


def _rank_main(rank, world, port, out_dir, case=None):
    import sys
    for p in (os.path.dirname(HERE), os.path.join(os.path.dirname(HERE), "montecarlox.jl_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    from mcx import parallel as P
    _run(P, case or CASE, P.DistributedBackend(), out_dir)
    dist.barrier()
    dist.destroy_process_group()


def _check_against_oracle(res, spins_ref, series, pos, stage, steps, acc, r0=0, r1=None):
    assert np.array_equal(res["series"], series)
    assert np.array_equal(res["pos"], pos)
    assert int(res["stage"][0]) == stage
    assert np.array_equal(res["steps"], steps) and np.array_equal(res["acc"], acc)
    assert np.array_equal(res["obs"], series[-1])
    r1 = len(spins_ref) if r1 is None else r1
    assert np.array_equal(res["spins"], np.concatenate(list(spins_ref[r0:r1]) + [np.zeros(0, np.int8)]))


def test_ladder_exchange_matches_oracle_exchange(mcxlib):
    """mcx_ladder_exchange (host, no GPU) against the oracle's exchange stage."""
    import ctypes as C
    from mcx import _lib as L
    rng = np.random.default_rng(5)
    for trial in range(40):
        n = int(rng.integers(2, 12))
        betas = np.sort(rng.uniform(0.1, 0.9, n))[::-1].copy()
        P = rng.integers(-3 * 64, 3 * 64, n).astype(np.int64)
        M = rng.integers(-64, 64, n).astype(np.int64)
        J, h = float(rng.choice([1.0, 0.5])), float(rng.choice([0.0, 0.3]))
        pos = rng.permutation(n).astype(np.int32)
        stage = int(rng.integers(0, 2))
        seed, ladder, t = int(rng.integers(0, 2 ** 63)), int(rng.integers(0, 4)), int(rng.integers(0, 2 ** 40))
        p_ref, st_ref = pos.copy(), stage
        s_ref, a_ref = np.zeros(n - 1, np.uint64), np.zeros(n - 1, np.uint64)
        x = (-(J * P.astype(np.float64))) - (h * M.astype(np.float64))
        st_ref = O.pt_exchange(betas, p_ref, st_ref, x, seed, ladder, t, s_ref, a_ref)
        st = C.c_int32(stage)
        s, a = np.zeros(n - 1, np.uint64), np.zeros(n - 1, np.uint64)
        assert L.load().mcx_ladder_exchange(n, betas.ctypes.data, P.ctypes.data, M.ctypes.data, J, h,
                                            pos.ctypes.data, C.byref(st), seed, ladder, t, s.ctypes.data,
                                            a.ctypes.data) == 0
        assert np.array_equal(pos, p_ref) and st.value == st_ref, trial
        assert np.array_equal(s, s_ref) and np.array_equal(a, a_ref)


def test_ladder_exchange_argument_errors(mcxlib):
    import ctypes as C
    from mcx import _lib as L
    b = np.array([0.3, 0.2, 0.1])
    P = np.zeros(3, np.int64)
    s, a = np.zeros(2, np.uint64), np.zeros(2, np.uint64)
    st = C.c_int32(0)
    bad = np.array([0, 0, 2], np.int32)  # not a permutation
    assert L.load().mcx_ladder_exchange(3, b.ctypes.data, P.ctypes.data, P.ctypes.data, 1.0, 0.0, bad.ctypes.data,
                                        C.byref(st), 1, 0, 0, s.ctypes.data, a.ctypes.data) != 0
    one = np.array([0], np.int32)
    assert L.load().mcx_ladder_exchange(1, b.ctypes.data, P.ctypes.data, P.ctypes.data, 1.0, 0.0, one.ctypes.data,
                                        C.byref(st), 1, 0, 0, s.ctypes.data, a.ctypes.data) != 0


def test_ladder_one_process_matches_oracle(mcxlib):
    from mcx import parallel as P
    c = CASE
    ref = oracle_ladder(c["L"], c["dim"], c["betas"], c["seed"], c["nsweeps"], c["every"], c["alg"])
    _check_against_oracle(_run(P, c, None), *ref)


def test_ladder_two_ranks(tmp_path):
    """Five replicas over two gloo ranks (2 + 3): both ranks hold the oracle's positions,
    stage, counters and series; each holds the oracle's spins of its own replicas."""
    mp = pytest.importorskip("torch.multiprocessing")
    c = CASE
    ref = oracle_ladder(c["L"], c["dim"], c["betas"], c["seed"], c["nsweeps"], c["every"], c["alg"])
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    n = len(c["betas"])
    for rank in (0, 1):
        res = {k: np.load(tmp_path / ("%s%d.npy" % (k, rank))) for k in
               ("series", "pos", "stage", "steps", "acc", "obs", "spins")}
        _check_against_oracle(res, *ref, r0=n * rank // 2, r1=n * (rank + 1) // 2)


@pytest.mark.parametrize("betas", [[0.30, 0.27, 0.245, 0.22, 0.2], [0.4, 0.2]])
def test_ladder_three_ranks(tmp_path, betas):
    """Uneven shares over three ranks (1 + 2 + 2 replicas, and 0 + 1 + 1 for a two-replica
    ladder): the same result on every rank as the oracle's single-process ladder."""
    mp = pytest.importorskip("torch.multiprocessing")
    c = dict(CASE, betas=betas)
    ref = oracle_ladder(c["L"], c["dim"], c["betas"], c["seed"], c["nsweeps"], c["every"], c["alg"])
    mp.spawn(_rank_main, args=(3, _free_port(), str(tmp_path), c), nprocs=3, join=True)
    n = len(betas)
    for rank in range(3):
        res = {k: np.load(tmp_path / ("%s%d.npy" % (k, rank))) for k in
               ("series", "pos", "stage", "steps", "acc", "obs", "spins")}
        _check_against_oracle(res, *ref, r0=n * rank // 3, r1=n * (rank + 1) // 3)  # rank 0 of 3 may hold none


def test_ladder_argument_errors(mcxlib):
    from mcx import parallel as P
    with pytest.raises(mcxlib.ArgumentError):
        P.DistributedLadder(4, [0.3], sweeper=OracleSweeper(4, 3, 0, 1))
    lad = P.DistributedLadder(4, [0.3, 0.2], sweeper=OracleSweeper(4, 3, 0, 2))
    with pytest.raises(mcxlib.ArgumentError):
        lad.sweep_(2, exchange_every=0)
    with pytest.raises(mcxlib.ArgumentError):
        lad.sweep_(2, alg="wolff")
    with pytest.raises(mcxlib.ArgumentError):
        lad.spins(5)


def test_ladder_without_record_matches(mcxlib):
    """Runs that keep no series (only the last sweep before each exchange is gathered)
    reach the same state as recorded runs, for several exchange intervals."""
    from mcx import parallel as P
    c = CASE
    for every in (1, 3):
        ref = oracle_ladder(c["L"], c["dim"], c["betas"], c["seed"], 10, every, "heatbath")
        lad = P.DistributedLadder(c["L"], c["betas"], dim=c["dim"], seed=c["seed"],
                                  sweeper=OracleSweeper(c["L"], c["dim"], 0, len(c["betas"])))
        lad.init_(c["seed"])
        assert lad.sweep_(7, alg="heatbath", exchange_every=every) is None
        lad.sweep_(3, alg="heatbath", exchange_every=every)
        assert np.array_equal(lad.positions, ref[2]) and lad.stage == ref[3]
        assert np.array_equal(lad.steps, ref[4]) and np.array_equal(lad.accepted, ref[5])
        assert np.array_equal(lad.observables(), ref[1][-1])
        for r in range(len(c["betas"])):
            assert np.array_equal(lad.spins(r), ref[0][r])

"""Processes as ranks (gloo, world size 2, CPU): the multicanonical exchange of
parallel_multicanonical.jl and the all-reduce of parallel_chains.jl over
torch.distributed, checked against a single-process computation with the oracle."""
import os
import socket

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import sys
    for p in (os.path.dirname(HERE), os.path.join(os.path.dirname(HERE), "montecarlox.jl_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    from mcx import parallel as P
    import oracle as O
    be = P.DistributedBackend()
    rng = np.random.default_rng(100 + rank)
    H = rng.integers(0, 50, size=33).astype(np.int64)      # this rank's visits
    lnw = rng.normal(size=33) if rank == 0 else np.zeros(33)
    np.save(os.path.join(out_dir, "H%d.npy" % rank), H)
    P.merge_histograms_(H, be)                               # root: sum of both
    if be.is_root():
        O.muca_update(lnw, H)                                # update!(ensemble) on the root
    P.distribute_logweight_(lnw, be)
    np.save(os.path.join(out_dir, "lnw%d.npy" % rank), lnw)
    t = np.array([1.5 + rank, 7.0 - rank])
    P.merge_(t, "max", be)
    np.save(os.path.join(out_dir, "max%d.npy" % rank), t)
    s = np.array([rank + 1], np.int64)
    P.merge_(s, "sum", be)
    np.save(os.path.join(out_dir, "sum%d.npy" % rank), s)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_multicanonical_exchange(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    import oracle as O
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    H0, H1 = np.load(tmp_path / "H0.npy"), np.load(tmp_path / "H1.npy")
    rng = np.random.default_rng(100)  # rank 0's draws: its histogram, then its weights
    rng.integers(0, 50, size=33)
    lnw = rng.normal(size=33)
    O.muca_update(lnw, H0 + H1)
    for r in (0, 1):
        assert np.array_equal(np.load(tmp_path / ("lnw%d.npy" % r)), lnw)
        assert np.array_equal(np.load(tmp_path / ("max%d.npy" % r)), [2.5, 7.0])
        assert np.array_equal(np.load(tmp_path / ("sum%d.npy" % r)), [3])


def test_backend_needs_a_process_group(mcxlib):
    from mcx import parallel as P
    with pytest.raises(mcxlib.ArgumentError):
        P.DistributedBackend()

"""Chains spread over processes (one per GPU): the MPI backend of the reference's
ParallelChains / ParallelMulticanonical restated over torch.distributed.

Reference (paths inside MonteCarloX.jl):
  update!(rx, x) (MPI backend)   src/algorithms/replica_exchange.jl:227-243 (pair exchange, Allgather)
  merge!(values, op, pc)         src/infrastructure/parallel_chains.jl:115-128 (Allreduce)
  merge_histograms!(pc)          src/algorithms/parallel_multicanonical.jl:31-52 (Reduce to root)
  distribute_logweight!(pc)      src/algorithms/parallel_multicanonical.jl:54-72 (Bcast from root)

Each process drives its own device objects; the only data exchanged are the int64
histograms and the FP64 log weights of a multicanonical iteration (and whatever a caller
merges).  The exchange goes through host memory, which works with the gloo backend on
CPU and with NCCL (tensors are moved to the process's GPU when the backend is NCCL).
Arguments may be device ensembles (MulticanonicalEnsemble / WangLandauEnsemble) or numpy
arrays, which are updated in place.
"""
import ctypes as C

import numpy as np

from . import ArgumentError

__all__ = ["DistributedBackend", "merge_", "merge_histograms_", "distribute_logweight_", "DistributedLadder"]

_OPS = {"sum": "SUM", "+": "SUM", "max": "MAX", "min": "MIN", "prod": "PRODUCT", "*": "PRODUCT"}


class DistributedBackend:
    """An initialised torch.distributed process group (default: the world) and the root
    rank that merges (the reference's MPIBackend(comm, root))."""

    def __init__(self, group=None, root=0):
        import torch.distributed as dist
        if not dist.is_available() or not dist.is_initialized():
            raise ArgumentError("torch.distributed is not initialised")
        self.group, self.root = group, int(root)
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)
        self.device = None
        if dist.get_backend(group) == "nccl":
            import torch
            self.device = torch.device("cuda", torch.cuda.current_device())

    def is_root(self):
        return self.rank == self.root

    def _tensor(self, arr):
        import torch
        t = torch.from_numpy(np.ascontiguousarray(arr))
        return t.to(self.device) if self.device is not None else t


def merge_(values, op, backend):
    """merge!(values, op, pc): all-reduce ``values`` (a numpy array, updated in place and
    returned) with op "sum", "max", "min" or "prod" over the processes."""
    import torch.distributed as dist
    if op not in _OPS:
        raise ArgumentError("unknown reduction %r" % (op,))
    arr = values if isinstance(values, np.ndarray) else np.asarray(values)
    t = backend._tensor(arr)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, _OPS[op]), group=backend.group)
    arr[...] = t.cpu().numpy()
    return arr


def _get(obj, what):
    if isinstance(obj, np.ndarray):
        return obj
    return getattr(obj, what)


def _set(obj, what, arr):
    if isinstance(obj, np.ndarray):
        obj[...] = arr
    else:
        setattr(obj, what, arr)


def merge_histograms_(ensemble, backend):
    """merge_histograms!(pc): the root receives the sum of every process's histogram
    (int64); the other processes keep theirs."""
    import torch.distributed as dist
    h = np.ascontiguousarray(_get(ensemble, "histogram"), np.int64)
    t = backend._tensor(h)
    dist.reduce(t, dst=backend.root, op=dist.ReduceOp.SUM, group=backend.group)
    if backend.is_root():
        _set(ensemble, "histogram", t.cpu().numpy())
    return ensemble


def distribute_logweight_(ensemble, backend):
    """distribute_logweight!(pc): every process takes the root's FP64 log weights."""
    import torch.distributed as dist
    lw = np.ascontiguousarray(_get(ensemble, "logweight"), np.float64)
    t = backend._tensor(lw)
    dist.broadcast(t, src=backend.root, group=backend.group)
    _set(ensemble, "logweight", t.cpu().numpy())
    return ensemble


class _DeviceSweeper:
    """The replicas r0 .. r1-1 of a ladder as device lattices of this process's GPU."""

    def __init__(self, L, dim, J, h, r0, r1, stream0=0, ctx=None):
        from . import Ising
        self.r0, self.s0 = r0, r0 + stream0  # replica r0 + i sweeps on stream s0 + i
        self.lattices = [Ising([int(L)] * int(dim), J=J, h=h, ctx=ctx) for _ in range(r0, r1)]

    def init(self, seed):
        from . import Philox, init_
        for i, lat in enumerate(self.lattices):
            init_(lat, "random", rng=Philox(seed, self.s0 + i))

    def spins(self, i):
        return self.lattices[i].spins

    def set_spins(self, i, values):
        self.lattices[i].spins = values

    def observables(self):
        from . import observables
        return np.array([observables(lat)[:2] for lat in self.lattices], np.int64).reshape(-1, 2)

    def sweep(self, betas, seed, t0, nsweeps, alg):
        """nsweeps sweeps of replica r0 + i at betas[i] on stream s0 + i from sweep t0;
        returns the (nsweeps, nlocal, 2) series of (pair sum, spin sum)."""
        from . import Glauber, HeatBath, Metropolis, Philox, sweep_batch_
        if not self.lattices:
            return np.zeros((nsweeps, 0, 2), np.int64)
        kind = {"metropolis": Metropolis, "glauber": Glauber, "heatbath": HeatBath}[alg]
        algs = [kind(Philox(seed, self.s0 + i, t0), beta=float(b)) for i, b in enumerate(betas)]
        obs = sweep_batch_(self.lattices, algs, nsweeps, record=True)
        return np.stack([o[:, :2] for o in obs], axis=1)

    def close(self):
        for lat in self.lattices:
            lat.close()
        self.lattices = []


class DistributedLadder:
    """One parallel-tempering ladder of Ising replicas spread over the processes of a group,
    one GPU each: the reference's ReplicaExchange with an MPI backend
    (src/algorithms/replica_exchange.jl:227-243 keeps one replica per rank and swaps
    packets between partners); here rank k of K keeps the replicas n*k//K .. n*(k+1)//K - 1.

    Replica r sweeps on its own stream, Philox(seed, stream0 + r) with the sweep index as
    counter, at the beta of its current ladder position (positions start as pos[r] = r).  Before an
    exchange step the ranks all-gather every replica's (pair sum, spin sum), and every rank
    takes the same exchange stage on the host (mcx_ladder_exchange: the uniforms and the
    arithmetic of the device exchange step).  Positions, stage and edge counters therefore
    agree on every rank, do not depend on the number of ranks, and equal a single-device
    ParallelTempering run of the same ladder (ladder index `ladder`, its replicas from global
    replica index `stream0` on, same seed).

    sweep_, observables and energies are collective: every rank of the group calls them.

    backend: a DistributedBackend (None: one process holds the whole ladder).
    sweeper: what sweeps this rank's replicas (default: device lattices on the current
    context); it provides init(seed), spins(i), set_spins(i, v), observables() and
    sweep(betas, seed, t0, nsweeps, alg) -> (nsweeps, nlocal, 2) series."""

    def __init__(self, L, betas, *, dim=3, J=1, h=0, seed=1000, ladder=0, stream0=0, backend=None, ctx=None,
                 sweeper=None):
        self.betas = np.ascontiguousarray(betas, np.float64)
        self.n = int(self.betas.size)
        if self.n < 2:
            raise ArgumentError("a ladder needs at least 2 replicas")
        self.L, self.dim, self.J, self.h = int(L), int(dim), float(J), float(h)
        self.seed, self.ladder = int(seed) & (2 ** 64 - 1), int(ladder)
        self.backend = backend
        rank, size = (backend.rank, backend.size) if backend is not None else (0, 1)
        self.bounds = [self.n * k // size for k in range(size + 1)]
        self.r0, self.r1 = self.bounds[rank], self.bounds[rank + 1]
        self.pos = np.arange(self.n, dtype=np.int32)
        self.stage = 0
        self.counter = 0  # next sweep index
        self.steps = np.zeros(self.n - 1, np.uint64)
        self.accepted = np.zeros(self.n - 1, np.uint64)
        self.stream0 = int(stream0)
        self.sweeper = sweeper if sweeper is not None else _DeviceSweeper(L, dim, J, h, self.r0, self.r1,
                                                                          self.stream0, ctx)

    # -- state ---------------------------------------------------------------
    def local_replicas(self):
        return range(self.r0, self.r1)

    def init_(self, seed):
        """init!(sys, :random) of every local replica r from Philox(seed, stream0 + r)."""
        self.sweeper.init(int(seed))

    def spins(self, r):
        return self.sweeper.spins(self._local(r))

    def set_spins_(self, r, values):
        self.sweeper.set_spins(self._local(r), values)

    def _local(self, r):
        if not self.r0 <= r < self.r1:
            raise ArgumentError("replica %d is not held by this process (%d..%d)" % (r, self.r0, self.r1 - 1))
        return r - self.r0

    @property
    def positions(self):
        """0-based ladder position of each replica (rx.indices - 1), the same on every rank."""
        return self.pos.copy()

    @property
    def indices(self):
        return self.pos + 1

    def observables(self):
        """(pair sum, spin sum) of every replica, gathered from all ranks: (n, 2) int64."""
        return self._gather(self.sweeper.observables()[None])[0]

    def energies(self):
        P = self.observables()
        return (-(self.J * P[:, 0].astype(np.float64))) - (self.h * P[:, 1].astype(np.float64))

    def acceptance_rates(self):
        return np.where(self.steps > 0, self.accepted / np.maximum(self.steps, 1), 0.0)

    # -- running -------------------------------------------------------------
    def _gather(self, local):
        """(k, nlocal, 2) per rank -> (k, n, 2) in replica order, on every rank."""
        if self.backend is None:
            return np.ascontiguousarray(local, np.int64)
        import torch
        import torch.distributed as dist
        k = local.shape[0]
        width = max(b - a for a, b in zip(self.bounds[:-1], self.bounds[1:]))
        pad = np.zeros((k, width, 2), np.int64)
        pad[:, :local.shape[1]] = local
        t = self.backend._tensor(pad)
        parts = [torch.empty_like(t) for _ in range(self.backend.size)]
        dist.all_gather(parts, t, group=self.backend.group)
        out = np.empty((k, self.n, 2), np.int64)
        for q, part in enumerate(parts):
            a, b = self.bounds[q], self.bounds[q + 1]
            out[:, a:b] = part.cpu().numpy()[:, :b - a]
        return out

    def _exchange(self, PM, sweep):
        from . import _check
        from . import _lib as L
        st = C.c_int32(self.stage)
        P = np.ascontiguousarray(PM[:, 0], np.int64)  # held for the call
        M = np.ascontiguousarray(PM[:, 1], np.int64)
        _check(L.load().mcx_ladder_exchange(self.n, self.betas.ctypes.data, P.ctypes.data, M.ctypes.data, self.J, self.h,
                                            self.pos.ctypes.data, C.byref(st), self.seed, self.ladder, int(sweep),
                                            self.steps.ctypes.data, self.accepted.ctypes.data))
        self.stage = st.value

    def sweep_(self, nsweeps, alg="metropolis", exchange_every=1, record=False):
        """`nsweeps` sweeps of every replica with an exchange stage after every
        `exchange_every`-th sweep (counting from sweep index 0, as mcx_pt_run does).
        Returns the (nsweeps, n, 2) series of (pair sum, spin sum) by replica if `record`
        (gathered on every rank)."""
        every = int(exchange_every)
        if every < 1:
            raise ArgumentError("exchange_every must be >= 1")
        if alg not in ("metropolis", "glauber", "heatbath"):
            raise ArgumentError("unknown algorithm %r" % (alg,))
        series = [] if record else None
        done = 0
        while done < nsweeps:
            t = self.counter
            k = min(nsweeps - done, every - (t % every))  # up to and including the next exchange
            betas = self.betas[self.pos[self.r0:self.r1]]
            local = self.sweeper.sweep(betas, self.seed, t, k, alg)
            self.counter += k
            done += k
            exch = self.counter % every == 0
            if record:
                series.append(self._gather(local))
            if exch:
                last = series[-1][-1] if record else self._gather(local[-1:])[0]
                self._exchange(last, self.counter - 1)
        return np.concatenate(series) if record and series else (np.zeros((0, self.n, 2), np.int64) if record else None)

    def close(self):
        self.sweeper.close()

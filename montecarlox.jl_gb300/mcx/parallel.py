"""Chains spread over processes (one per GPU): the MPI backend of the reference's
ParallelChains / ParallelMulticanonical restated over torch.distributed.

Reference (paths inside MonteCarloX.jl):
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
import numpy as np

from . import ArgumentError

__all__ = ["DistributedBackend", "merge_", "merge_histograms_", "distribute_logweight_"]

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

"""mcx_sweep_noalloc -- the sweep entry point that allocates no device memory.

Some callers cannot let a library allocate device memory while they run: a Julia
program whose GPU memory all belongs to CUDA.jl's pool, a PyTorch program using its
caching allocator, a service that reserved its HBM up front.  For them the library
keeps its per-sweep scratch in one fixed device array, and the caller passes its own
device buffers for the outputs.  This test calls the entry point through the C ABI
(with output buffers that PyTorch allocated) and checks it against mcx_sweep on a
twin lattice, bit for bit (integer results: tolerance 0), on two calls in a row.

The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    ("ising", [64, 64], 0, 0.4407, 0.0),   # Metropolis, 128-bit row path
    ("ising", [16, 16, 16], 2, 0.25, 0.0),  # HeatBath, 3-D
    ("bc", [32, 24], 0, 0.6, 1.0),          # Blume-Capel Metropolis
    ("ising", [12, 8], 1, 0.3, 0.0),        # Glauber, one site per thread
]


def _lattice(mcx, kind, L, D, ctx):
    if kind == "ising":
        return mcx.Ising(L, ctx=ctx)
    return mcx.BlumeCapel(L, D=D, ctx=ctx)


@pytest.mark.parametrize("kind,L,alg,beta,D", CASES)
def test_noalloc_matches_mcx_sweep(gpu, kind, L, alg, beta, D):
    import torch

    mcx = gpu
    lib = mcx._lib.load()
    fn = lib.mcx_sweep_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(mcx._lib.mcx_rng), C.c_int64, C.c_void_p,
                   C.c_void_p]
    ctx = mcx.Context()
    a = _lattice(mcx, kind, L, D, ctx)
    b = _lattice(mcx, kind, L, D, ctx)
    mcx.init_(a, "random", rng=mcx.Philox(11))
    mcx.init_(b, "random", rng=mcx.Philox(11))
    ra = mcx._lib.mcx_rng(99, 0, 3, 0)
    rb = mcx._lib.mcx_rng(99, 0, 3, 0)
    for nsweeps in (7, 12):  # two calls in a row, the second continuing the first
        obs_a = np.zeros((nsweeps, 3), np.int64)
        cnt = mcx._lib.mcx_counters(0, 0)
        mcx._check(lib.mcx_sweep(a.handle, alg, beta, C.byref(ra), nsweeps, obs_a.ctypes.data, C.byref(cnt)))
        obs_b = torch.full((nsweeps, 3), -1, dtype=torch.int64, device="cuda")
        acc_b = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        used0 = ctx.memory()[0]
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        mcx._check(fn(b.handle, alg, beta, C.byref(rb), nsweeps, obs_b.data_ptr(), acc_b.data_ptr()))
        ctx.sync()
        assert ctx.memory()[0] == used0  # nothing allocated through the context
        if nsweeps == 12:  # after the first call has loaded the kernels: no device allocation at all
            assert torch.cuda.mem_get_info()[0] == free0
        assert rb.counter == ra.counter
        assert np.array_equal(obs_b.cpu().numpy(), obs_a)
        assert int(acc_b.item()) == cnt.accepted
        assert np.array_equal(a.spins, b.spins)
        assert mcx.observables(a) == mcx.observables(b)
        with pytest.raises(mcx.ArgumentError):  # no stale series after a no-alloc call
            mcx._check(lib.mcx_read_series(b.handle, np.zeros(3, np.int64).ctypes.data, 1))
    b.close()
    a.close()


def test_noalloc_rejects_more_sweeps_than_its_scratch(gpu):
    mcx = gpu
    lib = mcx._lib.load()
    fn = lib.mcx_sweep_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(mcx._lib.mcx_rng), C.c_int64, C.c_void_p,
                   C.c_void_p]
    lat = mcx.Ising([16, 16])
    r = mcx._lib.mcx_rng(1, 0, 0, 0)
    with pytest.raises(mcx.ArgumentError):
        mcx._check(fn(lat.handle, 0, 0.4, C.byref(r), 4097, None, None))
    assert r.counter == 0

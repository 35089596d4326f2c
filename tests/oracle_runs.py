"""Oracle runs shared by several GPU parity tests (test infrastructure).

* ``oracle_pt``: a batch of parallel-tempering ladders swept and exchanged by the oracle,
  replica after replica (replica r, ladder after ladder, draws stream r).
* ``muca_walker_range``: oracle Multicanonical sweeps of walkers i0..i1-1 on one shared
  log-weight table; the histogram adds up over the walkers as merge_histograms! does
  (src/algorithms/parallel_multicanonical.jl:38-47).  A top-level function so that a
  ``spawn`` process pool can run ranges of walkers side by side.
"""
import hashlib

import numpy as np

import oracle as O

ALG = {"metropolis": O.METROPOLIS, "glauber": O.GLAUBER, "heatbath": O.HEATBATH}


def oracle_pt(ladders, dim, alg, seed, nsweeps, every, J=1.0, h=0.0):
    """Returns (spins per replica, series[nsweeps, R, 2], positions, stage, edge steps,
    edge accepted), the layout of mcx.pt.ParallelTempering."""
    reps = [(L, l, k) for l, (L, b) in enumerate(ladders) for k in range(len(b))]
    spins = [O.init_random(O.ISING, [L] * dim, seed, r) for r, (L, l, k) in enumerate(reps)]
    pos = [np.arange(len(b), dtype=np.int32) for _, b in ladders]
    steps = [np.zeros(len(b) - 1, np.uint64) for _, b in ladders]
    acc = [np.zeros(len(b) - 1, np.uint64) for _, b in ladders]
    members = [[r for r, rr in enumerate(reps) if rr[1] == l] for l in range(len(ladders))]
    stage = 0
    series = np.zeros((nsweeps, len(reps), 2), np.int64)
    for t in range(nsweeps):
        for r, (L, l, k) in enumerate(reps):
            beta = ladders[l][1][pos[l][k]]
            O.cb_sweep(spins[r], O.ISING, [L] * dim, ALG[alg], beta, seed, stream=r, sweep0=t, nsweeps=1, J=J, h=h,
                       record=False)
            P, M, _ = O.observables(spins[r], [L] * dim)
            series[t, r] = (P, M)
        if (t + 1) % every == 0:
            new_stage = stage
            for l, (L, b) in enumerate(ladders):
                x = np.array([(-(J * float(series[t, r, 0]))) - (h * float(series[t, r, 1])) for r in members[l]])
                new_stage = O.pt_exchange(np.array(b), pos[l], stage, x, seed, l, t, steps[l], acc[l])
            stage = new_stage
    positions = np.concatenate(pos)
    return spins, series, positions, stage, np.concatenate(steps), np.concatenate(acc)


def muca_walker_range(args):
    """Oracle Multicanonical sweeps of Blume-Capel walkers i0..i1-1 (init!(:random) from
    (seed, i), stream i) on the shared table ``lnw``.  Returns (H summed over the range,
    per walker (rc, steps, accepted, sha1 of the final spins, per-sweep series))."""
    L, D, (start, step, nb), lnw, seed, i0, i1, nsweeps = args
    H = np.zeros(nb, np.int64)
    out = []
    for i in range(i0, i1):
        s = O.init_random(O.BC, L, seed, i)
        rc, obs, st, ac = O.flathist_sweep(s, O.BC, L, O.MUCA, lnw, H, start, step, 0.0, seed, stream=i,
                                           nsweeps=nsweeps, D=D)
        out.append((rc, st, ac, hashlib.sha1(s.tobytes()).hexdigest(), obs))
    return H, out

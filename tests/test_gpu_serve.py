"""Serving: continuous batching, HBM-budget admission, same result alone and in the mix (GPU)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

JOBS = [
    dict(model="ising", L=(64, 64), kind="canonical", alg="metropolis", beta=0.44, seed=5, stream=0, nsweeps=37),
    dict(model="bc", L=(48, 40), kind="canonical", alg="heatbath", beta=0.6, D=1.0, seed=5, stream=1, nsweeps=23),
    dict(model="ising", L=(16, 24), kind="canonical", alg="glauber", beta=0.3, seed=9, stream=2, nsweeps=61),
    dict(model="ising", L=(32, 32), kind="multicanonical", beta=0.4, seed=5, stream=3, nsweeps=15,
         bins=(-2048, 4, 1025)),
    dict(model="bc", L=(16, 16), kind="multicanonical", beta=0.5, D=1.0, seed=5, stream=4, nsweeps=12,
         bins=(-256, 1, 1025)),
    dict(model="ising", L=(128, 64), kind="canonical", alg="metropolis", beta=0.6, h=0.25, seed=1, stream=5,
         nsweeps=19),
]


def _spec(j):
    j = dict(j)
    if j["kind"] == "multicanonical":
        start, step, nb = j["bins"]
        j["logweight"] = -j["beta"] * (start + step * np.arange(nb)).astype(np.float64)
    return j


def _snapshot(job):
    r = job.result
    return (r["state"], r["status"], r["pair_sum"], r["spin_sum"], r["spin2_sum"], r["attempts"], r["accepted"],
            job.series.tobytes(), job.spins.tobytes(),
            None if job.histogram is None else job.histogram.tobytes(),
            None if job.logweight is None else job.logweight.tobytes())


def test_same_result_alone_and_in_the_mix(gpu):
    from mcx.serve import Server
    alone = []
    for j in JOBS:
        srv = Server(chunk=7)
        job = srv.submit(spins=True, **_spec(j))
        srv.run_until_idle()
        assert srv.poll(job) is not None and job.result["state"] == 2
        alone.append(_snapshot(job))
        srv.close()
    # in the mix: staggered arrivals, a budget that holds only some jobs at once
    srv = Server(hbm_budget=30_000, max_jobs=4, chunk=5)
    jobs = []
    for k, j in enumerate(JOBS):
        jobs.append(srv.submit(spins=True, **_spec(j)))
        if k % 2 == 1:
            srv.step()
    srv.run_until_idle()
    st = srv.stats()
    assert st["peak_bytes"] <= 30_000 and st["jobs_done"] == len(JOBS)
    for job, ref in zip(jobs, alone):
        assert srv.poll(job) is not None
        assert _snapshot(job) == ref  # bit for bit


def test_canonical_job_matches_oracle(gpu):
    from mcx.serve import Server
    srv = Server(chunk=4)
    job = srv.submit(spins=True, **JOBS[0])
    srv.run_until_idle()
    srv.poll(job)
    L = [64, 64]
    s = O.init_random(O.ISING, L, 5, 0)
    obs, att, acc = O.cb_sweep(s, O.ISING, L, O.METROPOLIS, 0.44, 5, stream=0, nsweeps=37)
    assert np.array_equal(job.series, obs)
    assert np.array_equal(job.spins, s)
    assert (job.result["attempts"], job.result["accepted"]) == (att, acc)


def test_multicanonical_job_matches_oracle(gpu):
    from mcx.serve import Server
    spec = _spec(JOBS[3])
    srv = Server(chunk=6)
    job = srv.submit(spins=True, **spec)
    srv.run_until_idle()
    srv.poll(job)
    L = [32, 32]
    s = O.init_random(O.ISING, L, 5, 3)
    lnw = spec["logweight"].copy()
    H = np.zeros(len(lnw), np.int64)
    rc, obs, st, ac = O.flathist_sweep(s, O.ISING, L, O.MUCA, lnw, H, -2048, 4, 0.0, 5, stream=3, nsweeps=15)
    assert rc == O.OK
    assert np.array_equal(job.series, obs) and np.array_equal(job.spins, s)
    assert np.array_equal(job.histogram, H)
    assert (job.result["attempts"], job.result["accepted"]) == (st, ac)


def test_budget_rejects_oversized_job_and_cancel(gpu):
    from mcx.serve import Server
    srv = Server(hbm_budget=10_000, max_jobs=2, chunk=5)
    with pytest.raises(gpu.BudgetError):
        srv.submit(model="ising", L=(256, 256), nsweeps=10)
    small = srv.submit(model="ising", L=(16, 16), nsweeps=50)
    srv.cancel(small)
    srv.run_until_idle()
    assert srv.poll(small)["state"] == 3


# ------------------------------------------------------------------ resident loop --
def test_resident_loop_same_result_as_stepped_server(gpu):
    """The resident loop (one persistent kernel fed through the mailbox) gives every job the
    stepped server's result bit for bit, alone and in a mix that a small arena admits a few
    jobs at a time, with staggered arrivals."""
    from mcx.serve import Server
    alone = []
    for j in JOBS:
        srv = Server(chunk=7)
        job = srv.submit(spins=True, **_spec(j))
        srv.run_until_idle()
        srv.poll(job)
        alone.append(_snapshot(job))
        srv.close()
    srv = Server(hbm_budget=4 << 20, max_jobs=3, resident=True)
    info = srv.loop_info()
    assert info["resident"]
    jobs = []
    for k, j in enumerate(JOBS):
        jobs.append(srv.submit(spins=True, **_spec(j)))
        if k % 2 == 1:
            srv.step()
    srv.run_until_idle()
    st = srv.stats()
    assert st["jobs_done"] == len(JOBS) and st["peak_bytes"] <= 4 << 20
    for job, ref in zip(jobs, alone):
        assert srv.poll(job) is not None
        assert _snapshot(job) == ref
    assert srv.loop_info()["launches"] >= 1
    srv.close()


def test_resident_loop_leaves_when_idle_and_comes_back(gpu):
    """With a short idle limit the loop kernel leaves once it has nothing to run (status 2)
    and the next job launches it again; results are unaffected."""
    import time
    from mcx.serve import Server
    srv = Server(hbm_budget=1 << 20, max_jobs=4, resident=True, loop_limits=(1 << 24, 2000))
    a = srv.submit(spins=True, **JOBS[0])
    srv.run_until_idle()
    t0 = time.time()
    while srv.loop_info()["running"] and time.time() - t0 < 10:
        srv.step()
        time.sleep(0.001)
    info = srv.loop_info()
    assert not info["running"] and info["status"] == 2
    b = srv.submit(spins=True, **JOBS[2])
    srv.run_until_idle()
    assert srv.loop_info()["launches"] == info["launches"] + 1
    ref = Server(chunk=5)
    ra, rb = ref.submit(spins=True, **JOBS[0]), ref.submit(spins=True, **JOBS[2])
    ref.run_until_idle()
    for x, y in ((a, ra), (b, rb)):
        srv.poll(x)
        ref.poll(y)
        assert _snapshot(x) == _snapshot(y)
    srv.close()
    ref.close()


def test_resident_loop_cancel_and_mixed_sizes(gpu):
    """A long job cancelled while the loop runs it is dropped at the end of a round; the
    other jobs (a 512^2 lattice among 16^2 ones) finish with the oracle's results."""
    from mcx.serve import Server
    import time
    srv = Server(hbm_budget=128 << 20, max_jobs=8, resident=True)
    long = srv.submit(model="ising", L=(256, 256), nsweeps=2_000_000, seed=3, stream=9, record=False)
    small = [srv.submit(model="ising", L=(16, 16), nsweeps=40 + 7 * k, seed=4, stream=k, beta=0.5, spins=True)
             for k in range(5)]
    big = srv.submit(model="bc", L=(512, 512), D=1.0, beta=0.6, nsweeps=30, seed=4, stream=20, spins=True)
    t0 = time.time()
    done = 0
    while time.time() - t0 < 20:
        srv.step()
        r = _progress(srv, long)
        if r["sweeps_done"] > 100 and all(srv.poll(j) is not None for j in small + [big]):
            done = r["sweeps_done"]
            break
    info = srv.loop_info()
    srv.cancel(long)
    srv.run_until_idle()
    r = srv.poll(long)
    assert r["state"] == 3, (done, r["sweeps_done"], info, time.time() - t0)
    for k, job in enumerate(small):
        assert srv.poll(job)["state"] == 2
        s = O.init_random(O.ISING, [16, 16], 4, k)
        obs, att, acc = O.cb_sweep(s, O.ISING, [16, 16], O.METROPOLIS, 0.5, 4, stream=k, nsweeps=40 + 7 * k)
        assert np.array_equal(job.series, obs) and np.array_equal(job.spins, s)
        assert (job.result["attempts"], job.result["accepted"]) == (att, acc)
    assert srv.poll(big)["state"] == 2
    s = O.init_random(O.BC, [512, 512], 4, 20)
    obs, att, acc = O.cb_sweep(s, O.BC, [512, 512], O.METROPOLIS, 0.6, 4, stream=20, nsweeps=30, D=1.0)
    assert np.array_equal(big.series, obs) and np.array_equal(big.spins, s)
    srv.close()


def test_resident_loop_runs_small_jobs_many_sweeps_per_round(gpu):
    """Small jobs (a colour within one pass of a block) run several sweeps per round on blocks
    of their own: 16^2 Ising and 64^2 Blume-Capel jobs with thousands of sweeps, first beside a
    512^2 job (one sweep per round each) and then alone, finish in far fewer rounds than sweeps
    with the oracle's spins, series and counters."""
    from mcx.serve import Server
    srv = Server(hbm_budget=64 << 20, max_jobs=8, resident=True)
    specs = [dict(model="ising", L=(16, 16), nsweeps=3001 + 17 * k, seed=5, stream=k, beta=0.44) for k in range(3)]
    specs.append(dict(model="bc", L=(64, 64), D=1.0, nsweeps=777, seed=5, stream=9, beta=0.6))
    specs.append(dict(model="ising", L=(512, 512), nsweeps=40, seed=5, stream=11, beta=0.44))
    jobs = [srv.submit(spins=True, **sp) for sp in specs]
    srv.run_until_idle()
    assert srv.loop_info()["rounds"] < 1000
    for job, sp in zip(jobs, specs):
        assert srv.poll(job)["state"] == 2
        model = O.ISING if sp["model"] == "ising" else O.BC
        D = sp.get("D", 0.0)
        s = O.init_random(model, list(sp["L"]), 5, sp["stream"])
        obs, att, acc = O.cb_sweep(s, model, list(sp["L"]), O.METROPOLIS, sp["beta"], 5, stream=sp["stream"],
                                   nsweeps=sp["nsweeps"], D=D)
        assert np.array_equal(job.series, obs) and np.array_equal(job.spins, s), sp
        assert (job.result["attempts"], job.result["accepted"]) == (att, acc)
    srv.close()


def _progress(srv, job):
    import ctypes as C
    from mcx import _lib as L
    r = L.mcx_job_result()
    L.load().mcx_server_poll(srv.handle, job.id, C.byref(r))
    return {f: getattr(r, f) for f, _ in L.mcx_job_result._fields_}


def test_resident_loop_needs_a_budget(gpu):
    from mcx.serve import Server
    with pytest.raises(gpu.ArgumentError):
        Server(resident=True)

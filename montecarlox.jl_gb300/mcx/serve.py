"""Serving: continuous batching of simulation jobs on one GPU (mcx_server_* C ABI).

A job is a 2-D Ising or Blume-Capel lattice started with init!(sys, :random) from
its own (seed, stream) and run for `nsweeps` checkerboard sweeps, canonically
(Metropolis / Glauber / HeatBath at beta) or with fixed Multicanonical weights.
Jobs queue in arrival order, are admitted while the HBM budget and slots allow,
and every scheduling step advances all admitted jobs together.
"""
import ctypes as C
import math
import time

import numpy as np

from . import _lib as _L
from . import _check, default_context, ArgumentError, NotReadyError

__all__ = ["Server", "Job", "poisson_jobs", "run_load"]

_MODEL = {"ising": _L.ISING, "bc": _L.BLUME_CAPEL, "blume_capel": _L.BLUME_CAPEL}
_ALG = {"metropolis": _L.METROPOLIS, "glauber": _L.GLAUBER, "heatbath": _L.HEATBATH}


class Job:
    def __init__(self, server, spec, outputs):
        self.server = server
        self.spec = spec
        self.outputs = outputs  # keeps the host buffers alive until the job finishes
        self.id = None
        self.result = None

    @property
    def series(self):
        return self.outputs.get("series")

    @property
    def histogram(self):
        return self.outputs.get("histogram")

    @property
    def logweight(self):
        return self.outputs.get("logweight")

    @property
    def spins(self):
        return self.outputs.get("spins")


class Server:
    """Continuous batching of jobs.  ``resident=True`` runs the sweeps in one persistent
    device loop fed through a mailbox (mcx_server_start); ``step`` then only admits, arms
    and retires jobs.  The resident loop needs an HBM budget (its job arena)."""

    def __init__(self, hbm_budget=0, max_jobs=64, chunk=50, ctx=None, resident=False, loop_limits=None):
        self.ctx = ctx or default_context()
        h = C.c_void_p()
        _check(_L.load().mcx_server_create(self.ctx.handle, int(hbm_budget), int(max_jobs), int(chunk), C.byref(h)))
        self.handle = h
        self.jobs = {}
        if loop_limits is not None:
            _check(_L.load().mcx_server_set_loop_limits(self.handle, int(loop_limits[0]), int(loop_limits[1])))
        if resident:
            _check(_L.load().mcx_server_start(self.handle))

    def loop_info(self):
        """(resident, running, status, launches, rounds) of the resident loop."""
        r, run, st = C.c_int32(), C.c_int32(), C.c_uint32()
        la, ro = C.c_uint64(), C.c_uint64()
        _check(_L.load().mcx_server_loop_info(self.handle, C.byref(r), C.byref(run), C.byref(st), C.byref(la),
                                              C.byref(ro)))
        return {"resident": bool(r.value), "running": bool(run.value), "status": st.value,
                "launches": la.value, "rounds": ro.value}

    def stop(self, timeout_s=10.0):
        _check(_L.load().mcx_server_stop(self.handle, float(timeout_s)))

    def submit(self, *, model="ising", L=(64, 64), kind="canonical", alg="metropolis", beta=0.44, J=1.0, D=0.0,
               h=0.0, seed=0, stream=0, nsweeps=100, bins=None, logweight=None, record=True, spins=False):
        job = _L.mcx_job()
        job.model = _MODEL[model]
        job.dim = 2
        job.L[0], job.L[1], job.L[2] = int(L[0]), int(L[1]), 1
        job.kind = {"canonical": _L.JOB_CANONICAL, "multicanonical": _L.JOB_MULTICANONICAL}[kind]
        job.alg = _ALG[alg]
        job.beta, job.J, job.D, job.h = float(beta), float(J), float(D), float(h)
        job.seed, job.stream, job.nsweeps = int(seed), int(stream), int(nsweeps)
        outputs = {}
        if record:
            outputs["series"] = np.zeros((int(nsweeps), 3), np.int64)
            job.obs_series = outputs["series"].ctypes.data
        if spins:
            outputs["spins"] = np.zeros(int(L[0]) * int(L[1]), np.int8)
            job.final_spins = outputs["spins"].ctypes.data
        if kind == "multicanonical":
            if bins is None:
                raise ArgumentError("Multicanonical jobs need bins (start, step, nbins)")
            start, step, nb = bins
            job.bin_start, job.bin_step, job.nbins = int(start), int(step), int(nb)
            if logweight is not None:
                outputs["logweight_in"] = np.ascontiguousarray(logweight, np.float64)
                job.logweight = outputs["logweight_in"].ctypes.data
            outputs["histogram"] = np.zeros(int(nb), np.int64)
            outputs["logweight"] = np.zeros(int(nb), np.float64)
            job.histogram = outputs["histogram"].ctypes.data
            job.logweight_out = outputs["logweight"].ctypes.data
        j = Job(self, job, outputs)
        jid = C.c_uint64()
        _check(_L.load().mcx_server_submit(self.handle, C.byref(job), C.byref(jid)))
        j.id = jid.value
        self.jobs[j.id] = j
        return j

    def step(self):
        a, p = C.c_int32(), C.c_int32()
        _check(_L.load().mcx_server_step(self.handle, C.byref(a), C.byref(p)))
        return a.value, p.value

    def poll(self, job):
        r = _L.mcx_job_result()
        st = _L.load().mcx_server_poll(self.handle, job.id, C.byref(r))
        if st == _L.MCX_ERR_NOT_READY:
            return None
        _check(st)
        job.result = {f: getattr(r, f) for f, _ in _L.mcx_job_result._fields_}
        return job.result

    def cancel(self, job):
        _check(_L.load().mcx_server_cancel(self.handle, job.id))

    def stats(self):
        s = _L.mcx_server_stats()
        _check(_L.load().mcx_server_get_stats(self.handle, C.byref(s)))
        return {f: getattr(s, f) for f, _ in _L.mcx_server_stats._fields_}

    def run_until_idle(self):
        while True:
            a, p = self.step()
            if a == 0 and p == 0:
                return

    def close(self):
        if getattr(self, "handle", None):
            _L.load().mcx_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_jobs(n, *, rate=200.0, seed=11, L_range=(32, 2048), beta_range=(0.3, 0.6), sweeps_range=(1e3, 1e5),
                 muca_fraction=0.5, muca_L_max=None, muca_sweeps_max=None, models=("ising", "bc")):
    """Synthetic request stream: Poisson arrivals (mean `rate` per s), L log-uniform in
    L_range (rounded to a multiple of 8; Multicanonical jobs capped at muca_L_max),
    beta uniform, sweeps log-uniform (Multicanonical jobs capped at muca_sweeps_max),
    Metropolis or Multicanonical, Ising or Blume-Capel (D = 1)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        Lside = int(round(math.exp(rng.uniform(math.log(L_range[0]), math.log(L_range[1]))) / 8.0)) * 8
        Lside = max(8, Lside)
        sweeps = int(round(math.exp(rng.uniform(math.log(sweeps_range[0]), math.log(sweeps_range[1])))))
        model = models[int(rng.integers(len(models)))]
        kind = "multicanonical" if rng.uniform() < muca_fraction else "canonical"
        if kind == "multicanonical" and muca_L_max is not None:
            Lside = min(Lside, int(muca_L_max) // 8 * 8)
        if kind == "multicanonical" and muca_sweeps_max is not None:
            sweeps = min(sweeps, int(muca_sweeps_max))
        beta = float(rng.uniform(*beta_range))
        N = Lside * Lside
        spec = dict(model=model, L=(Lside, Lside), kind=kind, alg="metropolis", beta=beta, seed=int(seed),
                    stream=i, nsweeps=sweeps, D=1.0 if model == "bc" else 0.0)
        if kind == "multicanonical":
            if model == "ising":
                spec["bins"] = (-2 * N, 4, N + 1)
                centers = -2 * N + 4 * np.arange(N + 1)
            else:
                spec["bins"] = (-N, 1, 4 * N + 1)
                centers = -N + np.arange(4 * N + 1)
            spec["logweight"] = -beta * centers.astype(np.float64)  # canonical-like weights
        out.append((t, spec))
    return out


def run_load(server, stream, *, record=False):
    """Replay a request stream in wall-clock time: submit each request at its arrival
    time, keep stepping the server, collect latencies (arrival to completion)."""
    t0 = time.perf_counter()
    live = []
    done = []
    i = 0
    while i < len(stream) or live:
        now = time.perf_counter() - t0
        while i < len(stream) and stream[i][0] <= now:
            arr, spec = stream[i]
            job = server.submit(record=record, **spec)
            live.append((arr, job))
            i += 1
        if not live:
            time.sleep(max(0.0, stream[i][0] - (time.perf_counter() - t0)))
            continue
        server.step()
        still = []
        for arr, job in live:
            r = server.poll(job)
            if r is None:
                still.append((arr, job))
            else:
                done.append((arr, time.perf_counter() - t0, job))
        live = still
    lat = np.array([fin - arr for arr, fin, _ in done])
    attempts = sum(j.result["attempts"] for _, _, j in done)
    wall = time.perf_counter() - t0
    return {"jobs": len(done), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "wall_s": wall, "attempts": int(attempts),
            "attempts_per_ns": attempts / (wall * 1e9), "failed": sum(1 for _, _, j in done if j.result["state"] != 2)}

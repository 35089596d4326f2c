#!/usr/bin/env python
"""Spin-flip throughput on one GB300 (and N independent replicas on N GPUs).

Workload (the 2-D configuration the headline metric is quoted on): Ising, L=4096
periodic, J=1, h=0, int8 spins, +/-1 start from seed 7, Metropolis checkerboard
sweeps at beta=0.4407, energy and magnetisation recorded every sweep.  One step is
one mcx_sweep call of --sweeps-per-step sweeps.  The lattice (16 MiB) fits in L2,
so L2 is flushed (256 MiB write) between timed steps.  The int8 lattice runs each call
on a transient 64-sites-per-word copy (packed at the start of the call, unpacked at its
end, k_msc_metro half-sweeps).  --uniforms (default planes) selects how the sweeps draw
each site's 32-bit Metropolis uniform (mcx_lattice_set_uniforms): "planes" takes its top 8
bits from bit planes shared by 64 sites and the low 24 only where they decide, "site" one
Philox word per site (the stream of every other kernel); both forms are bit-exact against
their oracle restatement and sample the same distribution, and the line reports the other
form's rate beside the headline (site_uniforms / plane_uniforms).

  value      attempts/ns, CUDA events on the library's stream (torch's current stream is
             handed to the context); L2 is flushed before every timed step, so each step
             starts from HBM, and the 16 MiB lattice stays L2-resident across the sweeps of
             the step
  e2e        the same metric through the public C ABI with host buffers: every step
             uploads the lattice from pinned host memory (mcx_set_spins) and reads
             the per-sweep (pair, spin, spin2) series back (mcx_sweep obs_series)
  roofline   the half-sweep kernel: algorithmic bytes 1.5*N/8 per launch (reads both
             packed colour arrays, writes its own) over the average launch time (packing
             included), against HBM; and
             int_frac, the fraction of the integer-pipe roof (issue, ALU, FMA) that binds the
             kernel, from its per-launch instruction counts and the sampled SM clock
  cpu_baseline  the oracle's sequential random-site mode (the reference's
             spin_flip! order, FP64 exp decisions), one chain per host core

Further lines in the same JSON object (skipped with --no-extras), each timed on its own:
  small_lattice     the L=64 configuration (10^3 + 10^4 sweeps, one block) and one such
                    chain per SM in one batched call
  medium_lattice    256^2 / 128^2 / 32^3 / Blume-Capel 256^2 in one thread-block cluster,
                    and seven 256^2 chains in one batched call
  reweighting       log Z, <E>, <E^2> at 100 betas from a 4,194,305-bin ln g on the device
  batched_pt        256 3-D replicas in five ladders: persistent kernel against the plain form
  serving           the serving configuration (Poisson 200 / s, L 32-2048, 1e3-1e5 sweeps) on the
                    resident loop, and a saturated queue on the resident loop and the stepped
                    server (p50 / p99 latency, aggregate attempts/ns)
  flat_histogram    Blume-Capel L=1024 Multicanonical walkers, one per resident block, and a
                    fixed-budget Wang-Landau stage 1 (ln f = 1, flatness 0.8, one walker per SM)
  site_uniforms     the headline workload with the other uniforms form (per-site words when the
                    headline draws bit planes), with its kernel's integer-pipe fractions
  msc64             the headline workload on the 64-spins-per-word layout (the headline's uniforms)
  c2_matrix         the configured 2-D runs: Metropolis and Glauber at beta 0.30 / 0.4407 / 0.60
                    on int8 and MSC64, 10^4 sweeps each with the series, then U4 and binning errors,
                    with per-site and with bit-plane uniforms
  other_lattices    3-D Ising 256^3 (both uniforms forms), Ising heat bath and Blume-Capel Metropolis / heat bath on
                    4096^2, and the headline workload with packing off (the int8 words,
                    k_ising_strip, with its own roofline)
  general_graphs    4096^2 torus as IsingMatrix (Gaussian couplings) and as IsingGraph

`--impl reference` times that CPU path alone on every host core.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "montecarlox.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

L_SIDE = 4096
BETA = 0.4407
SEED = 7
METRIC = "spin-flip attempts/ns"
UNIT = "attempts/ns"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["mcx", "reference"], default="mcx")
    ap.add_argument("--sweeps-per-step", type=int, default=200)
    ap.add_argument("--uniforms", choices=["planes", "site"], default="planes",
                    help="how the headline sweeps draw their uniforms (mcx_lattice_set_uniforms)")
    ap.add_argument("--algorithm", choices=["metropolis", "glauber", "heatbath"], default="metropolis",
                    help="the headline workload's rule (the configured workload is Metropolis)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the parallel-tempering and serving lines")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="bounded CPU sample length")
    ap.add_argument("--profile", choices=["pt", "flathist", "serve", "graph", "graph_table", "lattice_small",
                                          "lattice_cluster"],
                    default=None,
                    help="run one short workload for a profiler capture and exit (no JSON line)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# DRAM bytes (read + write) of one k_ising_strip<2,16,false,true> half-sweep launch on the
# headline lattice, from one ncu capture (profiles/int_pipes_ising_strip_and_pt_persistent.md;
# ncu replays with flushed caches, so this is a cold launch: both colour arrays read once)
CB_TRAFFIC_PER_LAUNCH = 16810240

# The same for one k_msc_metro<2,*> launch (the headline workload's kernel: int8 lattices run
# multi-sweep calls on a transient 64-sites-per-word copy), per uniforms form,
# profiles/msc_metro_L4096.md and profiles/int_pipes_ising_strip_and_pt_persistent.md.
MSC_TRAFFIC_PER_LAUNCH = {("site", "metropolis"): 2136064, ("planes", "metropolis"): 2118400,
                          ("planes", "glauber"): 2123520, ("planes", "heatbath"): 2120960}

# Per-launch integer-pipe work of the headline kernels from one ncu capture each
# (profiles/int_pipes_ising_strip_and_pt_persistent.md): warp instructions, ALU-pipe warp
# instructions (2 cycles each on a sub-partition's ALU pipe) and FMA-pipe active cycles.
CB_PIPES = {"warp_inst": 7033664, "alu_inst": 3798288, "fma_cycles": 7453376, "per": "launch"}
MSC_PIPES = {("site", "metropolis"): {"warp_inst": 4686044, "alu_inst": 2143878, "fma_cycles": 6684336, "per": "launch"},
             ("planes", "metropolis"): {"warp_inst": 2712288, "alu_inst": 1276356, "fma_cycles": 2420152,
                                        "per": "launch"},
             ("planes", "glauber"): {"warp_inst": 3616731, "alu_inst": 1978005, "fma_cycles": 2560230, "per": "launch"},
             ("planes", "heatbath"): {"warp_inst": 3748500, "alu_inst": 2221129, "fma_cycles": 2761404, "per": "launch"}}


def headline_kernel(uniforms, algorithm):
    """The half-sweep kernel of the headline lattice for a uniforms form and rule."""
    if uniforms == "planes":
        return "k_msc_metro<2,true,%d>" % {"metropolis": 0, "glauber": 1, "heatbath": 2}[algorithm]
    return "k_msc_metro<2,false,0>" if algorithm == "metropolis" else "k_ising_strip (int8 words)"
PT_PIPES = {"warp_inst": 64528754 / 3, "alu_inst": 32555444 / 3, "fma_cycles": 67545556 / 3, "per": "sweep"}


def int_roof(pipes, seconds, sm_mhz, nsm):
    """Fractions of the integer roofs reached in `seconds` per launch (or sweep): issue
    (1 warp instruction per cycle per sub-partition), ALU pipe (2 cycles per instruction) and
    FMA pipe (the counted active cycles); int_frac is the largest, the pipe that binds."""
    cycles = nsm * 4 * sm_mhz * 1e6 * seconds
    issue = pipes["warp_inst"] / cycles
    alu = 2.0 * pipes["alu_inst"] / cycles
    fma = pipes["fma_cycles"] / cycles
    return {"int_frac": max(issue, alu, fma), "issue_frac": issue, "alu_frac": alu, "fma_frac": fma,
            "sm_mhz": sm_mhz, "counts_per": pipes["per"]}


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
            os.unlink(self.path)
        except Exception:
            return None
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_sample(seconds, nthreads, per_thread=None):
    """Oracle sequential random-site mode on `nthreads` chains, sized to ~`seconds` by a pilot
    run unless `per_thread` (attempts per chain) is given."""
    import oracle as O

    L = [L_SIDE, L_SIDE]
    if per_thread is None:
        pilot = 200_000
        t = O.bench_seq(O.ISING, L, O.METROPOLIS, BETA, SEED, nthreads, pilot)
        rate = nthreads * pilot / max(t, 1e-6)
        per_thread = max(pilot, int(rate * seconds / nthreads))
    t = O.bench_seq(O.ISING, L, O.METROPOLIS, BETA, SEED, nthreads, per_thread)
    return nthreads * per_thread / (t * 1e9), t, per_thread


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    ncores = os.cpu_count() or 1
    secs = max(1.0, min(5.0, 120.0 / max(1, args.steps + args.warmup)))
    vals, times, per = [], [], None
    for k in range(args.warmup + args.steps):
        v, t, per = cpu_sample(secs, ncores, per)  # sized by a pilot on the first step
        if k >= args.warmup:
            vals.append(v)
            times.append(t)
    value = statistics.mean(vals)
    sample = "%d host threads x %d sequential random-site Metropolis attempts on an L=%d lattice each" % (
        ncores, per, L_SIDE)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int8", "data": "synthetic", "impl": "reference",
        "config": {"workload": "ising2d_L4096_metropolis", "L": L_SIDE, "beta": BETA, "seed": SEED,
                   "order": "sequential random-site (spin_flip! order)", "precision": "fp64 exp decisions"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


PT_SIZES = [16, 24, 32, 48, 64]
PT_COUNTS = [52, 51, 51, 51, 51]


def bench_pt(torch, mcx, ctx, dev, flush, steps, warmup, sweeps_per_step=100, plain_sweeps=2):
    """3-D parallel tempering, 256 replicas of uneven size (L 16..64, ~51 each),
    geometric beta 0.20 -> 0.25 per size, exchange every sweep: the persistent batched
    form against the plain one-lattice-per-launch form (same results bit for bit)."""
    from mcx.pt import ParallelTempering, set_betas

    ladders = [(L, set_betas(n, 0.20, 0.25, ":geometric")) for L, n in zip(PT_SIZES, PT_COUNTS)]
    pt = ParallelTempering(ladders, dim=3, seed=SEED, ctx=ctx)
    pt.init_(SEED)
    default_schedule = pt.schedule[:3]
    tuned = pt.autotune_("metropolis", exchange_every=1, sweeps=20)  # state restored; results unchanged
    sites = sum(L ** 3 * n for L, n in zip(PT_SIZES, PT_COUNTS))
    stream = torch.cuda.current_stream(dev)
    out = {}
    for mode, nsw in (("persistent", sweeps_per_step), ("plain", plain_sweeps)):
        for _ in range(warmup):
            flush.zero_()
            pt.sweep_(nsw, mode=mode)
        torch.cuda.synchronize()
        l0 = ctx.launches()
        tot = 0.0
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            pt.sweep_(nsw, mode=mode)
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        out[mode] = {"attempts_per_ns": sites * nsw * steps / (tot * 1e6), "ms_per_sweep": tot / (nsw * steps),
                     "sweeps_per_step": nsw, "gpu_launches": ctx.launches() - l0}
    peak, _ = measured_peaks()
    per = out["persistent"]
    achieved = 3.0 * sites / (per["ms_per_sweep"] * 1e-3) / 1e9
    return {
        "workload": "pt3d_ising_256replicas_L16-64_exchange_every_sweep", "replicas": pt.nrep, "sites": sites,
        "persistent": per, "plain": out["plain"],
        "speedup_vs_plain": per["attempts_per_ns"] / out["plain"]["attempts_per_ns"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "alg_bytes_per_sweep": 3 * sites, "kernel": "k_pt_persistent<3,false,true>"},
        "exchange_acceptance": float(pt.acceptance_rate()),
        "schedule": {"default": list(default_schedule), "tuned": list(tuned[:3]),
                     "tuned_ns_per_attempt": tuned[3],
                     "fields": "blocks_per_sm, widest chunk (sites per thread), warp-split weights"},
    }


def bench_headline_form(torch, mcx, ctx, flush, steps, warmup, sweeps_per_step, layout, uniforms, nsm, sm_mhz):
    """The headline workload on `layout` with `uniforms` (the int8 layout on its transient
    packed copy, or the 64-spins-per-word layout itself): device-timed, L2 flushed between
    steps, with the half-sweep kernel's integer-pipe fractions."""
    L = [L_SIDE, L_SIDE]
    N = L_SIDE * L_SIDE
    lat = mcx.Ising(L, layout=layout, ctx=ctx)
    lat.set_uniforms(uniforms)
    mcx.init_(lat, "random", rng=mcx.Philox(SEED))
    alg = mcx.Metropolis(mcx.Philox(SEED), beta=BETA)
    lib = mcx._lib.load()

    def step():
        rng = alg.rng._c()
        mcx._check(lib.mcx_sweep(lat.handle, alg.ALG, BETA, mcx.C.byref(rng), sweeps_per_step, None, None))
        alg.rng.counter = rng.counter

    for _ in range(warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        step()
        e1.record()
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    lat.close()
    launch_s = tot * 1e-3 / (2 * sweeps_per_step * steps)
    return {"workload": "ising2d_L4096_metropolis_%s_%s_uniforms" % (layout, uniforms),
            "attempts_per_ns": N * sweeps_per_step * steps / (tot * 1e6), "ms_per_step": tot / steps,
            "sweeps_per_step": sweeps_per_step, "kernel": headline_kernel(uniforms, "metropolis"),
            "roofline": int_roof(MSC_PIPES[(uniforms, "metropolis")], launch_s, sm_mhz, nsm)}


def bench_int8_words(torch, mcx, ctx, flush, steps, warmup, sweeps_per_step, nsm, sm_mhz):
    """The headline workload with packing off (mcx_lattice_set_packing): every half-sweep on
    the int8 words (k_ising_strip, captured 64-sweep graphs), device-timed, L2 flushed."""
    L = [L_SIDE, L_SIDE]
    N = L_SIDE * L_SIDE
    lat = mcx.Ising(L, ctx=ctx)
    lat.set_packing(False)
    mcx.init_(lat, "random", rng=mcx.Philox(SEED))
    alg = mcx.Metropolis(mcx.Philox(SEED), beta=BETA)
    lib = mcx._lib.load()

    def step():
        rng = alg.rng._c()
        mcx._check(lib.mcx_sweep(lat.handle, alg.ALG, BETA, mcx.C.byref(rng), sweeps_per_step, None, None))
        alg.rng.counter = rng.counter

    for _ in range(warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        step()
        e1.record()
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    lat.close()
    launch_s = tot * 1e-3 / (2 * sweeps_per_step * steps)
    return {"workload": "ising2d_L4096_metropolis_int8_words", "attempts_per_ns": N * sweeps_per_step * steps / (tot * 1e6),
            "ms_per_step": tot / steps, "sweeps_per_step": sweeps_per_step, "kernel": "k_ising_strip<2,16,false,true>",
            "roofline": dict({"alg_bytes_per_launch": 1.5 * N, "achieved_gbs": 1.5 * N / launch_s / 1e9,
                              "traffic": CB_TRAFFIC_PER_LAUNCH}, **int_roof(CB_PIPES, launch_s, sm_mhz, nsm))}


def bench_c2_matrix(torch, mcx, ctx, sweeps=10000):
    """The 2-D L=4096 configuration as configured: Metropolis and Glauber at beta 0.30, 0.4407
    and 0.60, on the int8 and the MSC64 layout, seed 7, `sweeps` sweeps in one call with
    (pair, spin) recorded every sweep (CUDA events around the call, series copied back
    inside), then the Binder cumulant U4 (jackknife) and the binning error of the energy per
    site from the series, after the first tenth as thermalisation.  Every run with per-site
    uniforms, and again with bit-plane uniforms (keys ending in _planes)."""
    import numpy as np
    from mcx import analysis as A
    N = L_SIDE * L_SIDE
    out = {}
    for alg_name, kind in (("metropolis", mcx.Metropolis), ("glauber", mcx.Glauber)):
        for beta, layout, uniforms in [(b, l, u) for u in ("site", "planes") for b in (0.30, 0.4407, 0.60)
                                       for l in ("int8", "msc64")]:
            lat = mcx.Ising([L_SIDE, L_SIDE], layout=layout, ctx=ctx)
            lat.set_uniforms(uniforms)
            mcx.init_(lat, "random", rng=mcx.Philox(SEED))
            alg = kind(mcx.Philox(SEED), beta=beta)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            obs = mcx.sweep_(lat, alg, sweeps, record=True)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            lat.close()
            th = sweeps // 10
            e = -np.asarray(obs[th:, 0], np.float64) / N  # J = 1, h = 0: E = -(pair sum)
            m = np.asarray(obs[th:, 1], np.float64) / N
            u4, u4_err = A.binder_cumulant(m)
            out["%s_beta%.4g_%s%s" % (alg_name, beta, layout, "_planes" if uniforms == "planes" else "")] = {
                "attempts_per_ns": N * sweeps / (ms * 1e6), "ms": ms,
                "e_per_site": float(e.mean()), "e_err_binning": A.binning_error(e),
                "abs_m": float(np.abs(m).mean()), "u4": u4, "u4_err": u4_err,
                "acceptance": alg.accepted / float(N * sweeps) if alg_name == "metropolis" else None}
    return {"workload": "ising2d_L4096_seed7_%d_sweeps_record" % sweeps, "runs": out}


def bench_other_lattices(torch, mcx, ctx, flush, steps=3, warmup=3, sweeps_per_step=100):
    """Other single-lattice sweeps, device-timed, L2 flushed between steps: 3-D Ising 256^3
    (transient packed copy; per-site and bit-plane uniforms), Ising heat bath (int8 strip
    kernel; bit planes on the packed copy) and Blume-Capel (D = 1) Metropolis (per-site and
    plane proposal bits) / heat bath on the 4096^2 lattice (column-strip half-sweeps)."""
    lib = mcx._lib.load()
    def planes(lat):
        lat.set_uniforms("planes")
        return lat

    cases = [("ising3d_L256_metropolis", lambda: mcx.Ising([256, 256, 256], ctx=ctx), mcx.Metropolis, 0.2216),
             ("ising3d_L256_metropolis_plane_uniforms", lambda: planes(mcx.Ising([256, 256, 256], ctx=ctx)),
              mcx.Metropolis, 0.2216),
             ("ising2d_L4096_heatbath_plane_uniforms", lambda: planes(mcx.Ising([L_SIDE, L_SIDE], ctx=ctx)),
              mcx.HeatBath, BETA),
             ("ising2d_L4096_heatbath", lambda: mcx.Ising([L_SIDE, L_SIDE], ctx=ctx), mcx.HeatBath, BETA),
             ("bc2d_L4096_D1_metropolis", lambda: mcx.BlumeCapel([L_SIDE, L_SIDE], D=1.0, ctx=ctx), mcx.Metropolis,
              0.6),
             ("bc2d_L4096_D1_heatbath", lambda: mcx.BlumeCapel([L_SIDE, L_SIDE], D=1.0, ctx=ctx), mcx.HeatBath, 0.6),
             ("bc2d_L4096_D1_metropolis_plane_uniforms", lambda: planes(mcx.BlumeCapel([L_SIDE, L_SIDE], D=1.0, ctx=ctx)),
              mcx.Metropolis, 0.6)]
    out = {}
    for name, make, kind, beta in cases:
        lat = make()
        mcx.init_(lat, "random", rng=mcx.Philox(SEED))
        alg = kind(mcx.Philox(SEED), beta=beta)
        n = int(lat.N)

        def step():
            rng = alg.rng._c()
            mcx._check(lib.mcx_sweep(lat.handle, alg.ALG, beta, mcx.C.byref(rng), sweeps_per_step, None, None))
            alg.rng.counter = rng.counter

        for _ in range(warmup):
            flush.zero_()
            step()
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            step()
            e1.record()
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        lat.close()
        out[name] = {"attempts_per_ns": n * sweeps_per_step * steps / (tot * 1e6), "ms_per_step": tot / steps,
                     "sweeps_per_step": sweeps_per_step}
    return out


def bench_flathist(torch, mcx, ctx, dev, nwalkers=None, L=1024):
    """Multicanonical production on 2-D Blume-Capel L=1024, J=1, D=1 (integer energies,
    4,194,305 bins of FP64 ln g and int64 H shared by the walkers): one sweep of
    `nwalkers` independent walkers (one block of a producer and a consumer warp each).  The
    walker itself is serial, so the throughput comes from the number of walkers: by default
    one full wave, four walkers per SM (the resident limit of the walker kernel)."""
    from mcx import flathist as F
    if nwalkers is None:
        nwalkers = 4 * torch.cuda.get_device_properties(dev).multi_processor_count

    N = L * L
    walkers = []
    for i in range(nwalkers):
        s = mcx.BlumeCapel([L, L], D=1.0, ctx=ctx)
        mcx.init_(s, "random", rng=mcx.Philox(SEED, i))
        walkers.append(s)
    ens = F.MulticanonicalEnsemble((-N, 1, 4 * N + 1), ctx=ctx)
    alg = F.Multicanonical(mcx.Philox(SEED), ens)
    stream = torch.cuda.current_stream(dev)
    F.sweep_walkers_(walkers[:8], alg, 1)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    F.sweep_walkers_(walkers, alg, 1)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    for s in walkers:
        s.close()
    return {"workload": "bc2d_L1024_D1_muca_production_%d_walkers_1_sweep" % nwalkers, "walkers": nwalkers,
            "bins": 4 * N + 1, "attempts_per_ns": nwalkers * N / (ms * 1e6),
            "ns_per_attempt_per_walker": ms * 1e6 / N, "ms": ms}


def bench_wang_landau(torch, mcx, ctx, dev, nwalkers=None, L=1024, sweeps=24, check_every=6):
    """Wang-Landau stage 1 of the Blume-Capel configuration: L=1024, J=1, D=1, 4,194,305 bins,
    ln f = 1, flatness 0.8, one walker per SM, each with its own FP64 ln g and int64 H (the
    reference's WangLandau keeps one table per walker).  A fixed budget of `sweeps` sweeps,
    the flatness test on every walker's histogram every `check_every` sweeps.  Reports the
    sweep throughput, the cost of one flatness test of all walkers, and the flatness ratio
    min H / mean H over the visited bins reached at the end of the budget (the stage needs
    ratio >= 0.8 to end; a 1024^2 lattice needs far more sweeps than this budget)."""
    from mcx import flathist as F
    if nwalkers is None:
        nwalkers = torch.cuda.get_device_properties(dev).multi_processor_count
    N = L * L
    bins = (-N, 1, 4 * N + 1)
    walkers, algs = [], []
    for i in range(nwalkers):
        s = mcx.BlumeCapel([L, L], D=1.0, ctx=ctx)
        mcx.init_(s, "random", rng=mcx.Philox(SEED, i))
        walkers.append(s)
        algs.append(F.WangLandau(mcx.Philox(SEED, i), F.WangLandauEnsemble(bins, logf=1.0, ctx=ctx)))
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize()
    sweep_ms = check_ms = 0.0
    checks = 0
    ratios = []
    for k in range(sweeps // check_every):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        F.sweep_walkers_(walkers, algs, check_every)
        e1.record(stream)
        torch.cuda.synchronize()
        sweep_ms += e0.elapsed_time(e1)
        t0 = time.perf_counter()
        ratios = [F.flatness(a.ensemble, 0.8)[1] for a in algs]
        check_ms += (time.perf_counter() - t0) * 1e3
        checks += 1
    visited = int((algs[0].ensemble.histogram > 0).sum())
    for s in walkers:
        s.close()
    for a in algs:
        a.ensemble.close()
    done = (sweeps // check_every) * check_every
    return {"workload": "bc2d_L1024_D1_wang_landau_stage1_logf1_%d_walkers_%d_sweeps" % (nwalkers, done),
            "walkers": nwalkers, "bins": 4 * N + 1, "sweeps": done,
            "attempts_per_ns": nwalkers * N * done / (sweep_ms * 1e6), "ms_per_sweep": sweep_ms / done,
            "flatness_check_ms_all_walkers": check_ms / max(checks, 1),
            "flatness_ratio_mean": float(sum(ratios) / len(ratios)), "flatness_ratio_max": float(max(ratios)),
            "visited_bins_walker0": visited, "stage_flat": bool(max(ratios) >= 0.8)}


def bench_serve(mcx, ctx, njobs=120, nsat=100):
    """The serving configuration on the resident loop (one persistent kernel fed through a
    mailbox, jobs admitted into a 4 GiB arena, 64 slots).
      poisson:   Poisson arrivals at 200 / s (seed 11) of Metropolis or Multicanonical jobs on
                 2-D Ising / Blume-Capel, L log-uniform in [32, 2048], beta uniform in
                 [0.3, 0.6], sweeps log-uniform in [1e3, 1e5]; Multicanonical jobs (a quarter)
                 run a serial walker each and are capped at L = 64 and 2000 sweeps (a single
                 walker at L = 2048 and 1e5 sweeps would take hours at ~55 ns per attempt).
      saturated: `nsat` canonical jobs all queued at t = 0 (L in [32, 2048], sweeps in
                 [1e3, 1e4]) on the resident loop and on the stepped server, for the aggregate
                 throughput of continuous batching against the single-lattice rate.
    Latency = arrival to completion; attempts/ns = all attempts over the wall time."""
    from mcx.serve import Server, poisson_jobs, run_load
    out = {}
    stream = poisson_jobs(njobs, rate=200.0, seed=11, L_range=(32, 2048), sweeps_range=(1e3, 1e5),
                          muca_fraction=0.25, muca_L_max=64, muca_sweeps_max=2000)
    for mode in ("resident", "stepped"):
        srv = Server(hbm_budget=4 << 30, max_jobs=64, chunk=50, ctx=ctx, resident=mode == "resident")
        r = run_load(srv, stream)
        st = srv.stats()
        li = srv.loop_info()
        srv.close()
        r.update({"workload": "poisson200_seed11_ising_bc_L32-2048_sweeps1e3-1e5_muca_quarter_L<=64_sweeps<=2000",
                  "mode": "resident loop" if mode == "resident" else "stepped server", "peak_bytes": st["peak_bytes"],
                  "loop_launches": li["launches"]})
        out["poisson" if mode == "resident" else "poisson_stepped"] = r
    sat = poisson_jobs(nsat, rate=1e9, seed=12, L_range=(32, 2048), sweeps_range=(1e3, 1e4), muca_fraction=0.0)
    for mode in ("resident", "stepped"):
        srv = Server(hbm_budget=4 << 30, max_jobs=64, chunk=50, ctx=ctx, resident=mode == "resident")
        r = run_load(srv, sat)
        srv.close()
        r.update({"workload": "saturated_%d_canonical_jobs_L32-2048_sweeps1e3-1e4" % nsat,
                  "mode": "resident loop" if mode == "resident" else "stepped server"})
        out["saturated_" + mode] = r
    return out


def ctx_sms(torch):
    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def bench_small(torch, mcx, ctx, with_cpu, cpu_seconds):
    """The reference's own CPU-run configuration: 2-D Ising L=64, Metropolis at beta 0.4407,
    seed 42, 10^3 thermalisation sweeps then 10^4 sweeps with E and M recorded every sweep,
    each one library call (the second is timed with CUDA events on the context's stream,
    the per-sweep series copied back to the host inside the timed region); then one such
    chain per SM as independent chains in one batched call (mcx_sweep_batch)."""
    import numpy as np
    L = 64
    N = L * L
    lat = mcx.Ising([L, L], ctx=ctx)
    mcx.init_(lat, "random", rng=mcx.Philox(42))
    alg = mcx.Metropolis(mcx.Philox(42), beta=BETA)
    mcx.sweep_(lat, alg, 1000)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    obs = mcx.sweep_(lat, alg, 10000, record=True)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    lat.close()
    # the same chain replicated as independent chains (ParallelChains), one per SM, one call
    nch = ctx_sms(torch)
    chains = [mcx.Ising([L, L], ctx=ctx) for _ in range(nch)]
    for i, c in enumerate(chains):
        mcx.init_(c, "random", rng=mcx.Philox(42, i))
    calgs = [mcx.Metropolis(mcx.Philox(42, i), beta=BETA) for i in range(nch)]
    mcx.sweep_batch_(chains, calgs, 1000)
    torch.cuda.synchronize()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record()
    mcx.sweep_batch_(chains, calgs, 10000, record=True)
    e3.record()
    torch.cuda.synchronize()
    bms = e2.elapsed_time(e3)
    for c in chains:
        c.close()
    res = {"workload": "ising2d_L64_metropolis_1e3_therm_1e4_sweeps_record", "attempts_per_ns": N * 1e4 / (ms * 1e6),
           "batched_chains": nch, "batched_attempts_per_ns": nch * N * 1e4 / (bms * 1e6),
           "us_per_sweep": ms * 1e3 / 1e4, "kernel": "k_lattice_small<0,2,8,false,true> (256 threads)", "launches_per_call": 2,
           "series_rows": int(obs.shape[0])}
    if with_cpu:
        import oracle as O
        s = O.init_random(O.ISING, [L, L], 42)
        done, t, t0 = 0, 0.0, time.perf_counter()
        while t < cpu_seconds:
            O.seq_attempts(s, O.ISING, [L, L], O.METROPOLIS, BETA, 42, attempt0=done, nattempts=N * 100)
            done += N * 100
            t = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": done / t / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": "one chain of the sequential random-site order (spin_flip! with FP64 exp), "
                                         "L=64, %d attempts, %.1f s" % (done, t)}
    return res


def bench_medium(torch, mcx, ctx):
    """Medium lattices, one call of 1000 sweeps with E and M every sweep (CUDA events on the
    context's stream): every sweep of the call runs in one thread-block cluster."""
    import numpy as np
    res = []
    for dims, model, beta in (([256, 256], "ising", BETA), ([128, 128], "ising", BETA), ([32, 32, 32], "ising", 0.2216),
                              ([256, 256], "blume_capel", 0.6)):
        lat = mcx.Ising(dims, ctx=ctx) if model == "ising" else mcx.BlumeCapel(dims, D=1.0, ctx=ctx)
        mcx.init_(lat, "random", rng=mcx.Philox(SEED))
        alg = mcx.Metropolis(mcx.Philox(SEED), beta=beta)
        mcx.sweep_(lat, alg, 100)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        mcx.sweep_(lat, alg, 1000, record=True)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        N = int(np.prod(dims))
        res.append({"workload": "%s_%s_metropolis_1000_sweeps_record" % (model, "x".join(map(str, dims))),
                    "us_per_sweep": ms, "attempts_per_ns": N * 1000 / (ms * 1e6)})
        lat.close()
    # independent 256^2 chains (ParallelChains): one cluster each in one mcx_sweep_batch launch;
    # seven clusters of 16 CTAs run side by side on a GB300 (measured: 2.38 us per sweep for
    # seven chains, 2.88 for eight, where an eighth cluster shares SMs)
    nch = 7
    chains = [mcx.Ising([256, 256], ctx=ctx) for _ in range(nch)]
    for i, c in enumerate(chains):
        mcx.init_(c, "random", rng=mcx.Philox(SEED, i))
    calgs = [mcx.Metropolis(mcx.Philox(SEED, i), beta=BETA) for i in range(nch)]
    mcx.sweep_batch_(chains, calgs, 100)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    mcx.sweep_batch_(chains, calgs, 1000, record=True)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    res.append({"workload": "ising_256x256_metropolis_1000_sweeps_record_x%d_chains_one_call" % nch,
                "us_per_sweep": ms, "attempts_per_ns": nch * 65536 * 1000 / (ms * 1e6)})
    for c in chains:
        c.close()
    return {"kernel": "k_lattice_cluster (one cluster of up to 16 CTAs per lattice, one launch per call)", "lines": res}


def bench_reweight(torch, mcx, ctx):
    """Reweighting from a Multicanonical ln g on the device: the Blume-Capel L=1024 energy
    range (4N + 1 = 4,194,305 bins of width 1, a smooth synthetic ln g), log Z, <E> and
    <E^2> at 100 betas in one call (synchronous; wall time around it)."""
    import numpy as np
    from mcx import flathist as F
    N = 1024 * 1024
    nb = 4 * N + 1
    ens = F.MulticanonicalEnsemble((-N, 1, nb), ctx=ctx)
    x = np.linspace(-1.0, 1.0, nb)
    ens.logweight = -(N * np.log(3.0) * (1.0 - x * x))
    betas = np.linspace(0.3, 0.7, 100)
    ens.reweight(betas[:4])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ens.reweight(betas)
    dt = time.perf_counter() - t0
    ens.close()
    return {"workload": "reweight_bc_L1024_4194305_bins_100_betas", "ms_per_call": dt * 1e3,
            "bin_betas_per_ns": nb * len(betas) / (dt * 1e9), "kernel": "k_reweight_partial (FP64, mcx_exp)"}


def torus_csr(L, seed, per_entry):
    """CSR of the L x L periodic grid (first coordinate fastest, sorted rows) and, when
    per_entry, symmetric Gaussian couplings: the 2-D Edwards-Anderson spin glass."""
    import numpy as np
    n = L * L
    v = np.arange(n, dtype=np.int64)
    x, y = v % L, v // L
    right, left = y * L + (x + 1) % L, y * L + (x - 1) % L
    down, up = ((y + 1) % L) * L + x, ((y - 1) % L) * L + x
    nb = np.stack([right, left, down, up], 1)
    o = np.argsort(nb, axis=1)
    nb = np.take_along_axis(nb, o, 1)
    rowptr = np.arange(n + 1, dtype=np.int64) * 4
    J = None
    if per_entry:
        rng = np.random.default_rng(seed)
        jh, jv = rng.normal(size=n), rng.normal(size=n)  # edges (v, right(v)), (v, down(v))
        J = np.take_along_axis(np.stack([jh, jh[left], jv, jv[up]], 1), o, 1).reshape(-1)
    return rowptr, nb.reshape(-1).astype(np.int32), J


GRAPH_L = 4096
GRAPH_SWEEPS = 50


def bench_graph(torch, mcx, ctx, flush, steps, warmup, cpu_seconds, with_cpu):
    """General-graph sweeps on the 4096^2 torus: the Edwards-Anderson spin glass as an
    IsingMatrix (Gaussian J_ij, Metropolis at beta 1.0) and the ferromagnet as an
    IsingGraph (J = 1, beta 0.4407).  Device-timed, L2 flushed between steps; algorithmic
    bytes per site and sweep = 4 neighbours x (4 B index + 8 B coupling) + 4 neighbour
    spin reads + own spin read and write (IsingGraph: no couplings)."""
    from mcx.graph import IsingGraphDevice
    N = GRAPH_L * GRAPH_L
    out = {}
    for name, per_entry, beta, bps in (("ea2d_L4096_matrix_metropolis", True, 1.0, 4 * 12 + 4 + 2),
                                       ("ferro2d_L4096_graph_metropolis", False, BETA, 4 * 4 + 4 + 2)):
        rowptr, col, J = torus_csr(GRAPH_L, SEED, per_entry)
        sysd = IsingGraphDevice(rowptr, col, J, J=1.0, ctx=ctx)
        mcx.init_(sysd, "random", rng=mcx.Philox(SEED))
        alg = mcx.Metropolis(mcx.Philox(SEED), beta=beta)
        lib = mcx._lib.load()

        def step():
            rng = alg.rng._c()
            mcx._check(lib.mcx_graph_sweep(sysd.handle, alg.ALG, beta, mcx.C.byref(rng), GRAPH_SWEEPS, None, None,
                                           None))
            alg.rng.counter = rng.counter

        for _ in range(warmup):
            flush.zero_()
            step()
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            step()
            e1.record()
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        info = sysd.info()
        E_c, E_f = mcx.energy(sysd), mcx.energy(sysd, full=True)
        sysd.close()
        sweep_s = tot * 1e-3 / (steps * GRAPH_SWEEPS)
        peak, peak_kind = measured_peaks()
        achieved = bps * N / sweep_s / 1e9
        res = {"attempts_per_ns": N / sweep_s / 1e9, "ms_per_sweep": sweep_s * 1e3, "sweeps_per_step": GRAPH_SWEEPS,
               "colours": info["colours"], "kernel": "k_graph_class<0,%s>" % ("false,true,0" if per_entry else
                                                                             "true,false,0"),
               "alg_bytes_per_site": bps, "achieved_gbs": achieved, "peak_gbs": peak, "frac": achieved / peak,
               "peak_kind": peak_kind, "cached_minus_full_energy": E_c - E_f}
        if with_cpu and per_entry:
            import numpy as np

            import oracle as O
            Ls = 512
            rp, cl, Jv = torus_csr(Ls, SEED, True)
            g = O.Graph(rp, cl, Jv=Jv)
            sp = O.graph_init_random(Ls * Ls, SEED)
            ns, t, t0 = 0, 0.0, time.perf_counter()
            while t < cpu_seconds:
                O.graph_sweep(g, sp, O.METROPOLIS, beta, SEED, sweep0=ns, nsweeps=4)
                ns += 4
                t = time.perf_counter() - t0
            res["cpu_baseline"] = {"value": Ls * Ls * ns / t / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                                   "sample": "oracle colour-class sweeps (FP64 reference decisions) of a %dx%d "
                                             "Edwards-Anderson torus, %d sweeps, %.1f s, one thread" % (Ls, Ls, ns, t)}
        out[name] = res
    return out


def run_mcx(args):
    import numpy as np
    import torch

    import mcx

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    # an explicit stream shared by torch (flush, events) and the library: a context
    # given no stream (handle 0) would run on a private stream the events do not see
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx = mcx.Context(device=local, stream=stream.cuda_stream)
    assert ctx.stream == stream.cuda_stream
    S = args.sweeps_per_step
    L = [L_SIDE, L_SIDE]
    N = L_SIDE * L_SIDE
    lat = mcx.Ising(L, ctx=ctx)
    lat.set_uniforms(args.uniforms)
    mcx.init_(lat, "random", rng=mcx.Philox(SEED, rank))
    alg = {"metropolis": mcx.Metropolis, "glauber": mcx.Glauber, "heatbath": mcx.HeatBath}[args.algorithm](
        mcx.Philox(SEED, rank), beta=BETA)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def enqueue_step():
        rng = alg.rng._c()
        mcx._check(mcx._lib.load().mcx_sweep(lat.handle, alg.ALG, BETA, mcx.C.byref(rng), S, None, None))
        alg.rng.counter = rng.counter

    for _ in range(args.warmup):
        flush.zero_()
        enqueue_step()
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launches()
    barrier()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        enqueue_step()
        ev[k][1].record(stream)
    barrier()
    launches = ctx.launches() - launches0
    clk = clocks.stop()
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    if ws > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    attempts = N * S * args.steps * ws
    value = attempts / (total_ms * 1e6)

    # roofline of the half-sweep kernel (2 launches per sweep; the call's packing and
    # unpacking of the transient 64-sites-per-word copy are inside the average)
    avg_launch_s = total_ms * 1e-3 / (2 * S * args.steps)
    alg_bytes = 1.5 * N / 8
    achieved = alg_bytes / avg_launch_s / 1e9
    peak, peak_kind = measured_peaks()

    # end to end through the C ABI with pinned host buffers
    host_spins = torch.empty(N, dtype=torch.int8).pin_memory()
    host_spins.numpy()[:] = lat.spins
    host_obs = torch.empty((S, 3), dtype=torch.int64).pin_memory()
    lib = mcx._lib.load()
    e2e_times = []
    barrier()
    for k in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mcx._check(lib.mcx_set_spins(lat.handle, host_spins.data_ptr(), N))
        rng = alg.rng._c()
        cnt = mcx._lib.mcx_counters(0, 0)
        mcx._check(lib.mcx_sweep(lat.handle, alg.ALG, BETA, mcx.C.byref(rng), S, host_obs.data_ptr(),
                                 mcx.C.byref(cnt)))
        alg.rng.counter = rng.counter
        t1 = time.perf_counter()
        if k >= args.warmup:
            e2e_times.append(t1 - t0)
    e2e_s = sum(e2e_times)
    if ws > 1:
        t = torch.tensor([e2e_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = N * S * args.steps * ws / (e2e_s * 1e9)
    barrier()

    pt_res = srv_res = fh_res = msc_res = graph_res = small_res = med_res = rw_res = other_res = c2_res = None
    other_form = None
    nsm = ctx_sms(torch)
    if not args.no_extras:
        other_form = bench_headline_form(torch, mcx, ctx, flush, max(3, args.steps // 2), 3, S, "int8",
                                         "site" if args.uniforms == "planes" else "planes", nsm, 2070.0)
        small_res = bench_small(torch, mcx, ctx, rank == 0 and not args.no_cpu_baseline, min(args.cpu_seconds, 3.0))
        med_res = bench_medium(torch, mcx, ctx)
        rw_res = bench_reweight(torch, mcx, ctx)
        pt_res = bench_pt(torch, mcx, ctx, dev, flush, max(3, args.steps // 2), 2)
        srv_res = bench_serve(mcx, ctx)
        fh_res = bench_flathist(torch, mcx, ctx, dev)
        fh_res["wang_landau_stage1"] = bench_wang_landau(torch, mcx, ctx, dev)
        msc_res = bench_headline_form(torch, mcx, ctx, flush, max(3, args.steps // 2), 3, S, "msc64", args.uniforms,
                                      nsm, 2070.0)
        other_res = bench_other_lattices(torch, mcx, ctx, flush)
        c2_res = bench_c2_matrix(torch, mcx, ctx)
        other_res["ising2d_L4096_metropolis_int8_words"] = bench_int8_words(
            torch, mcx, ctx, flush, max(3, args.steps // 2), 3, S, ctx_sms(torch), (clk or {}).get("sm_mhz") or 2070.0)
        graph_res = bench_graph(torch, mcx, ctx, flush, max(3, args.steps // 4), 3, min(args.cpu_seconds, 5.0),
                                rank == 0 and not args.no_cpu_baseline)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        ncores = os.cpu_count() or 1
        v, t, per = cpu_sample(args.cpu_seconds, ncores)
        cpu = {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
               "sample": "%d host threads x %d sequential random-site Metropolis attempts (spin_flip! order, "
                         "FP64 exp) on an L=%d lattice each, %.1f s" % (ncores, per, L_SIDE, t)}
    tr = MSC_TRAFFIC_PER_LAUNCH.get((args.uniforms, args.algorithm))
    sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
    if pt_res:
        pt_res["roofline"].update(int_roof(PT_PIPES, pt_res["persistent"]["ms_per_sweep"] * 1e-3, sm_mhz, nsm))
    for r in (other_form, msc_res):  # the legs' fractions at the clock sampled in the timed region
        if r:
            r["roofline"] = int_roof(MSC_PIPES[(r["workload"].split("_")[-2], "metropolis")],
                                     r["ms_per_step"] * 1e-3 / (2 * S), sm_mhz, nsm)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int8", "data": "synthetic",
        "config": {"workload": "ising2d_L4096_%s_int8" % args.algorithm, "L": L_SIDE, "beta": BETA, "seed": SEED,
                   "layout": "int8 colour-split storage; each call sweeps a transient 64-sites-per-word copy "
                             "(packed at its start, unpacked at its end; mcx_lattice_set_packing)",
                   "uniforms": args.uniforms + (" (top 8 bits of each site's 32-bit uniform from bit planes "
                                                "shared by 64 sites, low 24 bits drawn where they decide; "
                                                "mcx_lattice_set_uniforms)" if args.uniforms == "planes" else
                                                " (one Philox word per site)"),
                   "sweeps_per_step": S, "record": "E,M every sweep",
                   "l2": "flushed between timed steps (256 MiB write)", "replicas_per_gpu": 1,
                   "parallelism": "replicas"},
        "roofline": dict({"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak, "traffic": tr, "peak_kind": peak_kind,
                          "kernel": headline_kernel(args.uniforms, args.algorithm),
                          "alg_bytes_per_launch": alg_bytes},
                         **(int_roof(MSC_PIPES[(args.uniforms, args.algorithm)], avg_launch_s, sm_mhz, nsm)
                            if (args.uniforms, args.algorithm) in MSC_PIPES else {})),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": N,
                "d2h_bytes_per_step": S * 3 * 8 + 8},
        "gpu_launches": launches,
        "clocks": clk,
        "cpu_baseline": cpu,
        "batched_pt": pt_res,
        "serving": srv_res,
        "flat_histogram": fh_res,
        ("site_uniforms" if args.uniforms == "planes" else "plane_uniforms"): other_form,
        "msc64": msc_res,
        "other_lattices": other_res,
        "c2_matrix": c2_res,
        "general_graphs": graph_res,
        "small_lattice": small_res,
        "medium_lattice": med_res,
        "reweighting": rw_res,
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_profile_target(args):
    """Short, fixed workloads for ncu captures (small enough for ~40 replays)."""
    import torch

    import mcx

    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = mcx.Context(device=0, stream=stream.cuda_stream)
    if args.profile == "pt":
        from mcx.pt import ParallelTempering, set_betas
        ladders = [(L, set_betas(n, 0.20, 0.25, ":geometric")) for L, n in zip(PT_SIZES, PT_COUNTS)]
        pt = ParallelTempering(ladders, dim=3, seed=SEED, ctx=ctx)
        pt.init_(SEED)
        pt.sweep_(3)
        pt.sweep_(10)
    elif args.profile == "flathist":
        from mcx import flathist as F
        L = [128, 128]
        walkers = []
        for i in range(64):
            s = mcx.BlumeCapel(L, D=1.0, ctx=ctx)
            mcx.init_(s, "random", rng=mcx.Philox(SEED, i))
            walkers.append(s)
        N = L[0] * L[1]
        ens = F.MulticanonicalEnsemble((-N, 1, 4 * N + 1), ctx=ctx)
        alg = F.Multicanonical(mcx.Philox(SEED), ens)
        F.sweep_walkers_(walkers, alg, 1)
        F.sweep_walkers_(walkers, alg, 2)
    elif args.profile == "serve":
        print(json.dumps(bench_serve(mcx, ctx)), flush=True)
    elif args.profile == "lattice_small":
        lat = mcx.Ising([64, 64], ctx=ctx)
        mcx.init_(lat, "random", rng=mcx.Philox(42))
        alg = mcx.Metropolis(mcx.Philox(42), beta=BETA)
        mcx.sweep_(lat, alg, 1000)
        mcx.sweep_(lat, alg, 10000, record=True)
    elif args.profile == "lattice_cluster":
        lat = mcx.Ising([256, 256], ctx=ctx)
        mcx.init_(lat, "random", rng=mcx.Philox(42))
        alg = mcx.Metropolis(mcx.Philox(42), beta=BETA)
        mcx.sweep_(lat, alg, 100)
        mcx.sweep_(lat, alg, 1000, record=True)
    elif args.profile in ("graph", "graph_table"):
        from mcx.graph import IsingGraphDevice
        # 4.2M sites; Gaussian couplings (0.25 GB of neighbour data) or one J (the table form)
        rowptr, col, J = torus_csr(2048, SEED, args.profile == "graph")
        sysd = IsingGraphDevice(rowptr, col, J, ctx=ctx)
        mcx.init_(sysd, "random", rng=mcx.Philox(SEED))
        alg = mcx.Metropolis(mcx.Philox(SEED), beta=1.0 if args.profile == "graph" else BETA)
        mcx.sweep_(sysd, alg, 2)
        mcx.sweep_(sysd, alg, 2)
    torch.cuda.synchronize()


def main():
    args = parse_args()
    if args.profile:
        run_profile_target(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_mcx(args)


if __name__ == "__main__":
    main()

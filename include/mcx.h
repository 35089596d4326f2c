/*
 * mcx.h -- C ABI of libmcx_cuda, the GB300 (sm_103a) spin-flip library.
 *
 * The library accelerates one hot path of MonteCarloX.jl + SpinSystems: the
 * single-spin-flip Metropolis / Glauber / HeatBath sweep over Ising and
 * Blume-Capel lattices, the Multicanonical / Wang-Landau histogram-and-weight
 * update, and the replica-exchange step of parallel tempering.  Every entry
 * point names the reference interface it replaces (paths inside MonteCarloX.jl).
 *
 * Conventions
 *   - Plain C types only; handles are opaque.  Device memory is owned by the
 *     library; host buffers are owned by the caller.
 *   - Spins cross the boundary in the SpinSystems linear order: site
 *     i = x + Lx*(y + Ly*z) (0-based), the Graphs.grid vertex order used by
 *     Ising(dims)/BlumeCapel(dims) (SpinSystems/src/ising.jl:413-424,
 *     SpinSystems/src/blume_capel.jl:500-511) and by IsingLatticeOptim (ising.jl:430-461).  Values are int8 in {-1,+1} (Ising)
 *     or {-1,0,+1} (Blume-Capel), as SpinSystems' `spins::Vector{Int8}`.
 *   - A context owns one CUDA stream; calls on one context are ordered on it.
 *     A context is not thread-safe; distinct contexts are independent.
 *   - Every call returns an mcx_status; mcx_last_error_string() gives details
 *     for the calling thread.  MCX_ERR_OUT_OF_RANGE is the BoundsError of the
 *     reference (an energy outside the histogram bins).
 *   - Lattices on the device need every side even and >= 4 (checkerboard order).
 */
#ifndef MCX_H
#define MCX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MCX_API __attribute__((visibility("default")))
#else
#define MCX_API
#endif

typedef enum mcx_status {
    MCX_OK = 0,
    MCX_ERR_INVALID_ARG = 1,
    MCX_ERR_OUT_OF_RANGE = 2, /* energy left the bin range (reference: BoundsError) */
    MCX_ERR_OOM = 3,          /* cudaMalloc failed                                  */
    MCX_ERR_BUDGET = 4,       /* the context's HBM budget would be exceeded          */
    MCX_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up                  */
    MCX_ERR_CUDA = 6,         /* any other CUDA runtime error                        */
    MCX_ERR_NOT_READY = 7,    /* a request has not finished yet                      */
    MCX_ERR_NOT_FOUND = 8     /* unknown request / handle                            */
} mcx_status;

typedef enum mcx_model { MCX_ISING = 0, MCX_BLUME_CAPEL = 1 } mcx_model;

/* Metropolis: src/algorithms/metropolis.jl:14-17, Glauber: :121-127,
 * HeatBath: src/algorithms/heat_bath.jl:11-17 + SpinSystems/src/ising.jl:43-58 /
 * SpinSystems/src/blume_capel.jl:61-85. */
typedef enum mcx_algorithm { MCX_METROPOLIS = 0, MCX_GLAUBER = 1, MCX_HEATBATH = 2 } mcx_algorithm;

/* INT8: one byte per site.  MSC64: 64 same-colour sites per uint64 word
 * (Ising only; needs Lx a multiple of 128). */
typedef enum mcx_layout { MCX_LAYOUT_INT8 = 0, MCX_LAYOUT_MSC64 = 1 } mcx_layout;

/* How checkerboard sweeps of a lattice draw the 32-bit uniform u that a site's
 * Metropolis decision u < threshold compares (both forms give every site an independent
 * uniform on [0, 2^32)).
 *   SITE (default): u is word e & 3 of one Philox4x32-10 block at counter e >> 2, e the
 *         site's index among the sites of its colour (one block per four sites).
 *   PLANES: the top 8 bits of u are bit planes: four Philox blocks per 64 same-colour
 *         sites give planes 0..7 (block j holds planes 2j and 2j+1 as two 64-bit words,
 *         bit b of a plane for site b of the 64), compared with the thresholds bit by bit
 *         for 64 sites at once; the low 24 bits come from a per-site block (like SITE,
 *         another counter purpose) and are drawn only for the sites whose top 8 bits equal
 *         their threshold's.  Applies to every Ising rule (Metropolis, Glauber, heat
 *         bath, with or without a field; all swept on 64-sites-per-word words).  On a
 *         Blume-Capel lattice PLANES replaces the proposal word (whose top bit is the
 *         proposal bit) by bit e & 63 of plane e >> 6, planes 2m and 2m+1 being words
 *         0 | 1 << 32 and 2 | 3 << 32 of one Philox block (one block per 128 sites); the
 *         acceptance words stay per site. */
typedef enum mcx_uniforms { MCX_UNIFORMS_SITE = 0, MCX_UNIFORMS_PLANES = 1 } mcx_uniforms;

/* Flat-histogram mode: Multicanonical (src/algorithms/multicanonical.jl) or
 * Wang-Landau (src/algorithms/wang_landau.jl). */
typedef enum mcx_flathist_mode { MCX_MUCA = 0, MCX_WANG_LANDAU = 1 } mcx_flathist_mode;

typedef struct mcx_config {
    int device;          /* CUDA device ordinal                                  */
    void* stream;        /* cudaStream_t to run on; NULL = a library-owned stream */
    uint64_t hbm_budget; /* bytes this context may allocate on the device; 0 = none */
} mcx_config;

/* Counter-based random stream: Philox4x32-10 keyed by `seed`; `counter` is the
 * next sweep index and advances by the number of sweeps run; `stream` separates
 * independent chains with the same seed.  Stands in for the `rng` field of the
 * reference's algorithm objects (src/algorithms/metropolis.jl:63-68). */
typedef struct mcx_rng {
    uint64_t seed;
    uint64_t counter;
    uint32_t stream;
    uint32_t reserved;
} mcx_rng;

/* `steps` / `accepted` of the reference's algorithm objects
 * (src/algorithms/importance_sampling.jl:23-28); accumulated, never reset. */
typedef struct mcx_counters {
    uint64_t attempts;
    uint64_t accepted;
} mcx_counters;

typedef struct mcx_ctx mcx_ctx;
typedef struct mcx_lattice mcx_lattice;
typedef struct mcx_flathist mcx_flathist;
typedef struct mcx_pt mcx_pt;
typedef struct mcx_server mcx_server;
typedef struct mcx_graph mcx_graph;

/* ---------------------------------------------------------------- errors -- */
MCX_API const char* mcx_status_string(mcx_status status);
MCX_API const char* mcx_last_error_string(void);
MCX_API int mcx_version(void);

/* --------------------------------------------------------------- context -- */
MCX_API mcx_status mcx_ctx_create(const mcx_config* config, mcx_ctx** out);
/* Releases the caller's handle.  Lattices, ensembles, ladders and servers created on
 * the context each hold it too: its stream and memory accounting are freed when the
 * last of them is destroyed, so the handles may be destroyed in any order. */
MCX_API mcx_status mcx_ctx_destroy(mcx_ctx* ctx);
MCX_API mcx_status mcx_sync(mcx_ctx* ctx);
MCX_API mcx_status mcx_ctx_stream(mcx_ctx* ctx, void** stream);
MCX_API mcx_status mcx_ctx_memory(mcx_ctx* ctx, uint64_t* used, uint64_t* budget);
/* Number of kernels this context has launched so far (for launch accounting). */
MCX_API mcx_status mcx_ctx_launches(mcx_ctx* ctx, uint64_t* launches);

/* --------------------------------------------------------------- lattice -- */
/* Replaces Ising(dims; J, periodic=true, h) (SpinSystems/src/ising.jl:413-424),
 * IsingLatticeOptim(Lx, Ly) (ising.jl:430-461) and BlumeCapel(dims; J, D, h)
 * (SpinSystems/src/blume_capel.jl:500-511).  All spins start at +1, like the
 * reference constructors. */
MCX_API mcx_status mcx_lattice_create(mcx_ctx* ctx, mcx_model model, int dim,
                                      const int32_t* L, mcx_layout layout, double J,
                                      double D, double h, mcx_lattice** out);
MCX_API mcx_status mcx_lattice_destroy(mcx_lattice* lat);
MCX_API mcx_status mcx_lattice_info(const mcx_lattice* lat, int64_t* nsites,
                                    int64_t* device_bytes);

/* The `spins` field of the reference systems (copy in / copy out). */
MCX_API mcx_status mcx_set_spins(mcx_lattice* lat, const int8_t* host, size_t n);
MCX_API mcx_status mcx_get_spins(mcx_lattice* lat, int8_t* host, size_t n);

/* init!(sys, :random; rng) (SpinSystems/src/ising.jl:60-78, SpinSystems/src/blume_capel.jl:87-109), fed by Philox. */
MCX_API mcx_status mcx_init_random(mcx_lattice* lat, uint64_t seed, uint32_t stream);
/* init!(sys, :up / :down / :zero): every site set to `value`. */
MCX_API mcx_status mcx_init_uniform(mcx_lattice* lat, int8_t value);

/* Cached bookkeeping of the reference systems (sum_pair_interactions without J,
 * sum_spins, sum_spins2; SpinSystems/src/ising.jl:430-438, SpinSystems/src/blume_capel.jl:117-126).  Waits for
 * the stream. */
MCX_API mcx_status mcx_observables(mcx_lattice* lat, int64_t* pair_sum, int64_t* spin_sum,
                                   int64_t* spin2_sum);
/* energy(sys; full=true) / magnetization(sys; full=true): recompute the bookkeeping
 * from the spins (SpinSystems/src/ising.jl:17-18, _recompute_cached! :141-159, :500-504); waits. */
MCX_API mcx_status mcx_recompute_observables(mcx_lattice* lat, int64_t* pair_sum,
                                             int64_t* spin_sum, int64_t* spin2_sum);
/* energy(sys), magnetization(sys) (SpinSystems/src/ising.jl:17-18, SpinSystems/src/blume_capel.jl:18-19):
 * E = -J*pair_sum - h*spin_sum + D*spin2_sum. */
MCX_API mcx_status mcx_energy(mcx_lattice* lat, double* energy, int64_t* magnetization);

/* N x spin_flip!(sys, alg) per sweep in checkerboard order, `nsweeps` sweeps
 * (replaces the user loop `for _ in 1:N; spin_flip!(sys, alg); end`, e.g.
 * docs/src/examples/spin_systems/importance_Ising2D.jl:105-122, over
 * spin_flip! SpinSystems/src/ising.jl:25-58 / SpinSystems/src/blume_capel.jl:41-85).
 *   obs_series: host int64[nsweeps*3] of (pair_sum, spin_sum, spin2_sum) after each
 *               sweep, or NULL.  counters: accumulated, or NULL.
 * With both NULL the call only enqueues work on the context stream. */
MCX_API mcx_status mcx_sweep(mcx_lattice* lat, mcx_algorithm alg, double beta,
                             mcx_rng* rng, int64_t nsweeps, int64_t* obs_series,
                             mcx_counters* counters);
/* Whether mcx_sweep may run calls of 16 sweeps or more of this int8 Ising lattice on a
 * transient 64-sites-per-word copy (Metropolis or Glauber without a field, Lx a multiple of 128,
 * above 524,288 sites): packed at the start of the call, unpacked at its end, N/8 bytes
 * of device memory on first use within the HBM budget.  Results are bit-identical either
 * way; the copy is faster.  Default on; off keeps every call on the int8 kernels. */
MCX_API mcx_status mcx_lattice_set_packing(mcx_lattice* lat, int32_t allow);
/* Selects the uniforms of later sweeps (mcx_uniforms; default SITE).  PLANES needs Lx a
 * multiple of 128 on an Ising lattice (MCX_ERR_INVALID_ARG otherwise); on the int8
 * layout its calls run on the transient 64-sites-per-word copy whatever their
 * length, so mcx_sweep returns MCX_ERR_INVALID_ARG with packing off and MCX_ERR_BUDGET /
 * MCX_ERR_OOM when the N/8-byte copy does not fit.  mcx_sweep_noalloc (int8 kernels
 * only) refuses such Ising calls; mcx_sweep_batch runs them one mcx_sweep per lattice.
 * Blume-Capel lattices of any size take PLANES on every launch form.  The form governs
 * mcx_sweep and mcx_sweep_batch; the flat-histogram walkers (mcx_flathist_sweep) and
 * mcx_spin_flip draw their own streams whatever it is.  The two forms give different
 * chains with the same distribution. */
MCX_API mcx_status mcx_lattice_set_uniforms(mcx_lattice* lat, int32_t form);
/* Times the admissible kernel shapes (sites per thread: 16, 8, 4) for this lattice
 * and algorithm on a scratch copy of the spins and keeps the fastest for later
 * mcx_sweep calls; results never depend on the choice.  chosen / ns_per_site may be
 * NULL. */
MCX_API mcx_status mcx_autotune(mcx_lattice* lat, mcx_algorithm alg, double beta,
                                int32_t* chosen, double* ns_per_site);
/* The sweeps of many independent lattices in one call (the chains of a ParallelChains
 * with a threads backend, src/infrastructure/parallel_chains.jl:99-105): lattice i runs
 * `nsweeps` sweeps at betas[i] on its own stream rngs[i] (advanced), with the results of
 * mcx_sweep(lats[i], alg, betas[i], &rngs[i], ...) bit for bit.  All lattices on one
 * context, one model and dimension.  int8 lattices of at most 16384 sites run in one
 * launch, one block per lattice; any other batch runs as one mcx_sweep per lattice.
 *   obs_series: n host pointers to int64[nsweeps*3] (or NULL entries), or NULL.
 *   counters:   n accumulated counters, or NULL. */
MCX_API mcx_status mcx_sweep_batch(mcx_lattice** lats, int32_t n, mcx_algorithm alg,
                                   const double* betas, mcx_rng* rngs, int64_t nsweeps,
                                   int64_t** obs_series, mcx_counters* counters);
/* `nattempts` x spin_flip!(sys, alg) in the reference's own order: each attempt picks a
 * uniformly random site (pick_site, SpinSystems/src/abstractions.jl:19) and decides with the
 * reference's FP64 rule (Ising: SpinSystems/src/ising.jl:25-58; Blume-Capel:
 * SpinSystems/src/blume_capel.jl:41-85; accept!: src/algorithms/importance_sampling.jl:80-85,
 * src/algorithms/metropolis.jl:121-127), the probabilities computed on the host with the C
 * library's exp.  Attempt a = rng->counter + k draws Philox4x32-10(seed, (a lo, a hi, 5<<24,
 * stream)): site ((w0<<32)|w1) mod N, U = u53(w2, w3); Blume-Capel Metropolis / Glauber
 * proposals take the top bit of word 0 of (a lo, a hi, 6<<24, stream).  rng->counter advances
 * by nattempts.  Serial by nature (one thread applies the attempts in order): a single-site
 * call for code written around spin_flip!, not a substitute for mcx_sweep.  Updates the cached
 * bookkeeping; counters (accumulated; HeatBath: accepted = spins that changed) may be NULL,
 * in which case the call only enqueues work. */
MCX_API mcx_status mcx_spin_flip(mcx_lattice* lat, mcx_algorithm alg, double beta, mcx_rng* rng,
                                 int64_t nattempts, mcx_counters* counters);
/* Copy the per-sweep series of the last mcx_sweep call (first n sweeps). */
MCX_API mcx_status mcx_read_series(mcx_lattice* lat, int64_t* obs_series, int64_t n);


/* --------------------------------------------------------- flat histogram -- */
/* A 1-D integer binning [start, start + step*nbins) of the total energy with an FP64
 * log-weight table (ln g) and an int64 visit histogram: the BinnedObject pair of
 * MulticanonicalEnsemble / WangLandauEnsemble (src/ensembles/multicanonical.jl:1-23,
 * src/ensembles/wang_landau.jl:1-21, src/infrastructure/binned_object.jl:13-24).
 * The bin of E is div(E - start, step) (truncating); bins outside [0, nbins) are the
 * reference's BoundsError.  ln g starts at 0, H at 0. */
MCX_API mcx_status mcx_flathist_create(mcx_ctx* ctx, int64_t start, int64_t step, int64_t nbins,
                                       mcx_flathist** out);
MCX_API mcx_status mcx_flathist_destroy(mcx_flathist* fh);
MCX_API mcx_status mcx_flathist_set_logweight(mcx_flathist* fh, const double* host, int64_t n);
MCX_API mcx_status mcx_flathist_get_logweight(mcx_flathist* fh, double* host, int64_t n);
MCX_API mcx_status mcx_flathist_set_histogram(mcx_flathist* fh, const int64_t* host, int64_t n);
MCX_API mcx_status mcx_flathist_get_histogram(mcx_flathist* fh, int64_t* host, int64_t n);
/* reset!(::Multicanonical) histogram part (src/algorithms/multicanonical.jl:27-33): H := 0. */
MCX_API mcx_status mcx_flathist_reset(mcx_flathist* fh);
/* Reweighting on the device from the ensemble's log density of states ln g = -logweight
 * (replaces distribution_from_logdos / log_sum, src/infrastructure/utils.jl:54-105, and the
 * energy moments of the reweighted distribution): for each betas[k] (nbeta in 1..65535),
 * over the bins whose w_b = ln g_b - beta E_b is finite (E_b the bin centres),
 * logz[k] = log sum exp(w_b), mean_e[k] = <E>, mean_e2[k] = <E^2>.  dist (may be NULL;
 * dist_len = nbins) receives exp(w_b - logz[0]) at betas[0], 0 on bins that are not finite.
 * FP64 throughout, deterministic; MCX_ERR_INVALID_ARG when no bin is finite. */
MCX_API mcx_status mcx_flathist_reweight(mcx_flathist* fh, const double* betas, int32_t nbeta, double* logz,
                                         double* mean_e, double* mean_e2, double* dist, int64_t dist_len);
/* update!(::MulticanonicalEnsemble; mode=:simple) (src/ensembles/multicanonical.jl:32-43):
 * ln g[b] -= log(H[b]) where H[b] > 0. */
MCX_API mcx_status mcx_flathist_update_muca(mcx_flathist* fh);
/* Wang-Landau flatness (the reference has none; Wang & Landau 2001): marks every bin
 * with H > 0 as visited (the mark persists across resets), then is_flat = min H >=
 * threshold * mean H over the visited bins; ratio = min H / mean H. */
MCX_API mcx_status mcx_flathist_flatness(mcx_flathist* fh, double threshold, int* is_flat,
                                         double* ratio);
/* The visited-bin marks of the flatness test (for checkpoint / resume). */
MCX_API mcx_status mcx_flathist_get_visited(mcx_flathist* fh, uint8_t* host, int64_t n);
MCX_API mcx_status mcx_flathist_set_visited(mcx_flathist* fh, const uint8_t* host, int64_t n);
/* merge_histograms! (src/algorithms/parallel_multicanonical.jl:38-47): dst.H += src[i].H. */
MCX_API mcx_status mcx_flathist_merge(mcx_flathist* dst, mcx_flathist* const* src, int nsrc);
/* distribute_logweight! (parallel_multicanonical.jl:59-68): dst.lnw := src.lnw. */
MCX_API mcx_status mcx_flathist_copy_logweight(mcx_flathist* dst, const mcx_flathist* src);
/* `nsweeps` checkerboard sweeps of N importance-sampling spin flips
 * (SpinSystems/src/ising.jl:25-33, SpinSystems/src/blume_capel.jl:41-50) for each of `nwalkers` walkers, with
 * accept!(alg, E_new, E_old) of a Multicanonical (importance_sampling.jl:69-78) or
 * Wang-Landau (src/algorithms/wang_landau.jl:29-37) algorithm; the decision lr > 0 || U < exp(lr)
 * is evaluated as log(U) < lr.  fhs: one table shared by all walkers (nfh = 1;
 * Multicanonical only: H adds up over walkers like merge_histograms!) or one per
 * walker (nfh = nwalkers).  Walker i draws from rngs[i].  Lattices must be int8, of
 * one shape and model, with integer J, D, h.  A walker whose energy leaves the bins
 * stops at that attempt with its counters unchanged; the call then returns
 * MCX_ERR_OUT_OF_RANGE.  The per-sweep (pair, spin, spin2) series of each walker is
 * readable with mcx_read_series. */
MCX_API mcx_status mcx_flathist_sweep(mcx_lattice* const* lattices, int nwalkers,
                                      mcx_flathist* const* fhs, int nfh, mcx_flathist_mode mode,
                                      double logf, mcx_rng* rngs, int64_t nsweeps,
                                      mcx_counters* counters);

/* ------------------------------------------------------ parallel tempering -- */
/* Batched replica exchange over `nladders` independent ladders: ladder l holds
 * nreplicas[l] Ising replicas (J, h) of side sides[l] (dim 2 or 3, side a multiple
 * of 8) at the inverse temperatures betas[...] listed ladder after ladder by ladder
 * position.  Replaces ParallelTempering(betas; seed, rng)
 * (src/algorithms/parallel_tempering.jl:24-53) over ReplicaExchange
 * (src/algorithms/replica_exchange.jl:13-19, 52-58) with one system per replica.
 * Replica r (0-based, ladder after ladder) draws its sweep stream with stream id r. */
typedef enum mcx_pt_mode {
    MCX_PT_PERSISTENT = 0, /* one cooperative launch for all sweeps of all replicas */
    MCX_PT_PLAIN = 1       /* one launch per replica and colour, one per exchange   */
} mcx_pt_mode;

MCX_API mcx_status mcx_pt_create(mcx_ctx* ctx, int dim, int nladders, const int32_t* sides,
                                 const int32_t* nreplicas, const double* betas, double J,
                                 double h, mcx_pt** out);
MCX_API mcx_status mcx_pt_destroy(mcx_pt* pt);
MCX_API mcx_status mcx_pt_info(const mcx_pt* pt, int32_t* nreplicas, int64_t* sites,
                               int64_t* device_bytes);
/* init!(sys, :random) of every replica (replica r uses stream r). */
MCX_API mcx_status mcx_pt_init_random(mcx_pt* pt, uint64_t seed);
MCX_API mcx_status mcx_pt_set_spins(mcx_pt* pt, int32_t replica, const int8_t* host, size_t n);
MCX_API mcx_status mcx_pt_get_spins(mcx_pt* pt, int32_t replica, int8_t* host, size_t n);
/* `nsweeps` checkerboard sweeps of every replica at its current ladder beta; after
 * every sweep t with (t+1) % exchange_every == 0, update!(rx, energies)
 * (replica_exchange.jl:158-178) on every ladder.  series: host
 * int64[nsweeps][nreplicas][2] of (pair_sum, spin_sum) after each sweep, or NULL. */
MCX_API mcx_status mcx_pt_run(mcx_pt* pt, mcx_algorithm alg, mcx_rng* rng, int64_t nsweeps,
                              int32_t exchange_every, mcx_pt_mode mode, int64_t* series);
/* index(rx) (replica_exchange.jl:48-50), 0-based: ladder position of each replica;
 * and the stage. */
MCX_API mcx_status mcx_pt_indices(mcx_pt* pt, int32_t* positions, int32_t* stage);
/* rx.steps / rx.accepted per ladder edge, ladder after ladder (n_l - 1 each). */
MCX_API mcx_status mcx_pt_exchange_counters(mcx_pt* pt, uint64_t* steps, uint64_t* accepted);
/* Restore ladder positions (a permutation within every ladder), the stage and the
 * edge counters, e.g. from a checkpoint (src/infrastructure/checkpointing.jl:95-100). */
MCX_API mcx_status mcx_pt_set_indices(mcx_pt* pt, const int32_t* positions, int32_t stage);
MCX_API mcx_status mcx_pt_set_exchange_counters(mcx_pt* pt, const uint64_t* steps,
                                                const uint64_t* accepted);
/* Cached (pair_sum, spin_sum) of every replica. */
MCX_API mcx_status mcx_pt_observables(mcx_pt* pt, int64_t* pair_sum, int64_t* spin_sum);
/* Series kept by mcx_pt_run on the device: 0 (default) only when the caller asks for it,
 * one column per replica; 1 always, per replica; 2 always, one column per global ladder
 * position (the energy trace at each fixed beta, as optimize_exchange_interval! groups
 * samples by ladder index, src/algorithms/parallel_tempering.jl:83-135).  With 2 the
 * `series` output of mcx_pt_run is in position order too. */
MCX_API mcx_status mcx_pt_set_record(mcx_pt* pt, int32_t record);
/* integrated_autocorrelation_times of the columns of the last run's device series:
 * quantity 0 energy (-J pair - h spin), 1 magnetization; per column under the batch
 * rules below (taus[nreplicas], NaN for skipped columns). */
MCX_API mcx_status mcx_pt_tau_int(mcx_pt* pt, int quantity, int64_t min_points, int64_t max_lag,
                                  double c, double* taus);
/* Accepted spin flips of every replica during the last mcx_pt_run. */
MCX_API mcx_status mcx_pt_replica_accepted(mcx_pt* pt, uint64_t* accepted);
/* Schedule of the persistent form (results never depend on it): blocks_per_sm in
 * 1..max_blocks_per_sm (0 = the maximum, the default), the co-resident blocks per SM of the
 * cooperative launch; vcap 16, 8 or 4, the widest chunk of same-colour sites a thread sweeps
 * (a replica takes the widest of 16, 8, 4 that divides its rows and is at most vcap; default
 * 16); weights 0, 1 or 2, the per-site costs (16-, 8-, 4-site chunks) by which warps are
 * handed to replicas: (1, 1.15, 1.4) (default), (1, 1, 1), (1, 1.3, 1.8).  No counterpart in
 * the reference, whose replicas run on threads or MPI ranks. */
MCX_API mcx_status mcx_pt_set_schedule(mcx_pt* pt, int32_t blocks_per_sm, int32_t vcap, int32_t weights);
MCX_API mcx_status mcx_pt_get_schedule(const mcx_pt* pt, int32_t* blocks_per_sm, int32_t* vcap, int32_t* weights,
                                       int32_t* max_blocks_per_sm);
/* Times every schedule (blocks per SM x vcap 16 / 8 x weights) with `sweeps` persistent sweeps
 * of the ladder's own state and keeps the fastest; the spins, cached observables, positions,
 * stage and counters are restored afterwards, the caller's rng is not used, and later runs give
 * the same results as without tuning.  Outputs may be NULL; ns_per_attempt is the chosen
 * schedule's host-timed cost per spin-flip attempt. */
MCX_API mcx_status mcx_pt_autotune(mcx_pt* pt, mcx_algorithm alg, int32_t exchange_every, int32_t sweeps,
                                   int32_t* blocks_per_sm, int32_t* vcap, int32_t* weights,
                                   double* ns_per_attempt);
/* Poll limit of the grid barrier waits (default 2^24 polls of ~100 ns). */
MCX_API mcx_status mcx_pt_set_wait_limit(mcx_pt* pt, int64_t polls);
/* Failure-detection check: a bounded wait on a device flag that nothing sets;
 * returns MCX_ERR_TIMEOUT after `polls` polls, with the context still usable. */
MCX_API mcx_status mcx_wait_flag_test(mcx_ctx* ctx, int64_t polls);
/* One exchange stage of one ladder of n replicas, on the host, for a ladder whose
 * replicas are swept by several processes (replaces update!(rx, xs) / update!(rx, x),
 * src/algorithms/replica_exchange.jl:158-178 and :227-243, with attempt_exchange_pair!
 * :124-136).  betas by ladder position; pair_sum / spin_sum / pos by replica (pos a
 * permutation of 0..n-1, updated in place); *stage 0 tries pairs (0,1), (2,3), ... and 1
 * tries (1,2), (3,4), ..., then flips; steps / accepted by lower position of each edge
 * (n - 1 entries, incremented).  The uniforms are those of the device exchange step for
 * (seed, ladder, sweep), so the positions equal a single-device mcx_pt_run on the same
 * ladder.  Needs no GPU. */
MCX_API mcx_status mcx_ladder_exchange(int32_t n, const double* betas, const int64_t* pair_sum,
                                       const int64_t* spin_sum, double J, double h, int32_t* pos,
                                       int32_t* stage, uint64_t seed, int32_t ladder, uint64_t sweep,
                                       uint64_t* steps, uint64_t* accepted);

/* ----------------------------------------------------------------- serving -- */
/* Continuous batching of simulation jobs (no counterpart in the reference, whose
 * users run one loop per system).  A job is a 2-D Ising or Blume-Capel lattice
 * started with init!(sys, :random) from (seed, stream) and run for nsweeps
 * checkerboard sweeps, canonically (alg, beta) or with fixed Multicanonical weights
 * over integer energy bins.  Jobs are admitted in arrival order while the server's
 * HBM budget and job slots allow, stay on the device until they finish, and share
 * every launch with the other active jobs.  A job's result does not depend on the
 * other jobs in the mix. */
typedef enum mcx_job_kind { MCX_JOB_CANONICAL = 0, MCX_JOB_MULTICANONICAL = 1 } mcx_job_kind;

typedef struct mcx_job {
    int32_t model;   /* mcx_model */
    int32_t dim;     /* 2 */
    int32_t L[3];    /* sides, multiples of 8 */
    int32_t kind;    /* mcx_job_kind */
    int32_t alg;     /* mcx_algorithm (canonical jobs) */
    int32_t reserved0;
    double beta, J, D, h;
    uint64_t seed;
    uint32_t stream;
    uint32_t reserved1;
    int64_t nsweeps;
    /* Multicanonical jobs: bins and initial log-weights (copied at submit, may be NULL) */
    int64_t bin_start, bin_step, nbins;
    const double* logweight;
    /* caller-owned host outputs, filled when the job finishes (each may be NULL) */
    int64_t* obs_series;    /* int64[nsweeps*3]: (pair, spin, spin2) after each sweep */
    int64_t* histogram;     /* int64[nbins] (Multicanonical) */
    double* logweight_out;  /* double[nbins] (Multicanonical) */
    int8_t* final_spins;    /* int8[L0*L1] in SpinSystems order */
} mcx_job;

typedef struct mcx_job_result {
    int32_t state;   /* 0 queued, 1 running, 2 done, 3 cancelled, 4 failed */
    int32_t status;  /* mcx_status of the job (MCX_ERR_OUT_OF_RANGE: left the bins) */
    int64_t pair_sum, spin_sum, spin2_sum;
    uint64_t attempts, accepted;
    int64_t sweeps_done;
    double submit_s, admit_s, finish_s; /* server clock, seconds since creation */
} mcx_job_result;

typedef struct mcx_server_stats {
    int32_t active, pending;
    uint64_t iterations, jobs_done, attempts_done;
    uint64_t bytes_in_use, peak_bytes;
    double now_s;
} mcx_server_stats;

/* hbm_budget: bytes the server's jobs may hold at once (0 = no limit); max_jobs: job
 * slots; chunk_sweeps: sweeps every active job advances per step. */
MCX_API mcx_status mcx_server_create(mcx_ctx* ctx, uint64_t hbm_budget, int32_t max_jobs,
                                     int32_t chunk_sweeps, mcx_server** out);
MCX_API mcx_status mcx_server_destroy(mcx_server* server);
/* Queue a job (MCX_ERR_BUDGET if it alone exceeds the budget). */
MCX_API mcx_status mcx_server_submit(mcx_server* server, const mcx_job* job, uint64_t* job_id);
/* One scheduling iteration: admit, advance every active job one chunk, retire. */
MCX_API mcx_status mcx_server_step(mcx_server* server, int32_t* active, int32_t* pending);
/* MCX_ERR_NOT_READY while queued or running; MCX_OK with the result once finished. */
MCX_API mcx_status mcx_server_poll(mcx_server* server, uint64_t job_id, mcx_job_result* result);
MCX_API mcx_status mcx_server_cancel(mcx_server* server, uint64_t job_id);
MCX_API mcx_status mcx_server_get_stats(mcx_server* server, mcx_server_stats* stats);
/* Switches a new server (before its first job is admitted) to the resident loop: one
 * persistent kernel on the device runs a sweep of every admitted canonical job per round,
 * takes newly admitted jobs from a mailbox in pinned host memory between rounds and
 * publishes finished ones there, so mcx_server_step no longer launches sweeps or waits for
 * the device: it admits jobs into a device arena of exactly hbm_budget bytes (allocated
 * here; no device allocation or free happens while the loop runs), arms them, retires the
 * finished ones, and launches the loop again when it has left for lack of work.
 * Multicanonical jobs run as walker launches on their own stream beside the loop.  Results
 * are those of the stepped server bit for bit.  Needs hbm_budget > 0 and max_jobs <= 256.
 * Every device wait is bounded: a grid barrier gives up after the spin limit (the next step
 * returns MCX_ERR_TIMEOUT and the affected jobs fail with it), and a round with nothing to
 * run waits at most the idle limit before the kernel leaves. */
MCX_API mcx_status mcx_server_start(mcx_server* server);
/* Asks the resident loop to leave at the end of its round and waits at most timeout_s
 * seconds (MCX_ERR_TIMEOUT); jobs still armed stay unfinished. */
MCX_API mcx_status mcx_server_stop(mcx_server* server, double timeout_s);
/* Bounds of the resident loop's waits: spin_polls per grid barrier (polls of ~0.1 us,
 * default 2^24) and idle_polls (polls of ~1 us, default 100000) before it leaves when it
 * has nothing to run; idle_polls * 100 < spin_polls. */
MCX_API mcx_status mcx_server_set_loop_limits(mcx_server* server, int64_t spin_polls, int64_t idle_polls);
/* Resident loop state: resident (started), running, status of the last launch (0 running,
 * 1 stopped, 2 left idle, 3 barrier timeout), launches so far, rounds of the current launch. */
MCX_API mcx_status mcx_server_loop_info(mcx_server* server, int32_t* resident, int32_t* running, uint32_t* status,
                                        uint64_t* launches, uint64_t* rounds);
/* The host side's bounded wait on a word the device (or another thread) writes: MCX_OK once
 * *flag >= target, MCX_ERR_TIMEOUT after `polls` polls sleeping sleep_ns each.  Needs no GPU. */
MCX_API mcx_status mcx_poll_flag(const uint32_t* flag, uint32_t target, int64_t polls, int64_t sleep_ns);

/* ------------------------------------------------------- general graphs -- */
/* Ising models on an arbitrary neighbour list: IsingGraph (one coupling J over a graph,
 * SpinSystems/src/ising.jl:86-139) and IsingMatrix (a symmetric sparse coupling
 * matrix J_ij, ising.jl:221-292, also what Ising(graph, Jvec) builds, :391-411), each
 * with no field, a uniform field h or a field per site (h::Vector).
 *   n:        number of sites (vertices), 0-based.
 *   rowptr:   int64[n+1], col: int32[rowptr[n]] -- row v lists the neighbours of v in
 *             strictly increasing order (the order of Graphs.neighbors and of the
 *             rowval of a SparseMatrixCSC); diagonal entries are skipped, like the
 *             j != i test of ising.jl:294-304.  Every off-diagonal (v, u) needs its
 *             (u, v) with the same coupling, else MCX_ERR_INVALID_ARG (the reference's
 *             AssertionError, ising.jl:252-263).
 *   coupling: float64[rowptr[n]] per entry (IsingMatrix), or NULL: every edge has J
 *             (IsingGraph).
 *   field:    float64[n] per site, or NULL: the uniform field h (0 = no field).
 * All spins start at +1.  Sites are updated in colour classes of a first-fit colouring
 * (in vertex order, each site the smallest colour its lower-numbered neighbours leave
 * free); one sweep visits every site once, class by class. */
MCX_API mcx_status mcx_graph_create(mcx_ctx* ctx, int64_t n, const int64_t* rowptr,
                                    const int32_t* col, const double* coupling, double J,
                                    const double* field, double h, mcx_graph** out);
/* BlumeCapelGraph(graph, J, D; h) / BlumeCapelMatrix(J, D; h) (SpinSystems/src/
 * blume_capel.jl:154-190, :328-360, factory :467-511): the same neighbour lists, spins in
 * {-1, 0, 1} (all +1 at start), E = -pair - field + D sum s^2.  Sweeps: Metropolis /
 * Glauber propose one of the two other states (_propose_state, :21-30) from bit 0 of the
 * low word of the site's uniform; the heat bath draws from the three Boltzmann weights
 * with r = u z (:61-85). */
MCX_API mcx_status mcx_bcgraph_create(mcx_ctx* ctx, int64_t n, const int64_t* rowptr,
                                      const int32_t* col, const double* coupling, double J,
                                      double D, const double* field, double h, mcx_graph** out);
MCX_API mcx_status mcx_graph_destroy(mcx_graph* g);
/* n sites, colour classes, stored neighbour entries (padding included), device bytes;
 * any pointer may be NULL. */
MCX_API mcx_status mcx_graph_info(const mcx_graph* g, int64_t* nsites, int32_t* colours,
                                  int64_t* entries, int64_t* device_bytes);
/* The colour of every site (int32[n]). */
MCX_API mcx_status mcx_graph_colours(const mcx_graph* g, int32_t* colour, size_t n);
/* The `spins` field (copy in / copy out, vertex order); values must be +1 or -1. */
MCX_API mcx_status mcx_graph_set_spins(mcx_graph* g, const int8_t* host, size_t n);
MCX_API mcx_status mcx_graph_get_spins(mcx_graph* g, int8_t* host, size_t n);
/* init!(sys, :random; rng) (ising.jl:60-78), fed by Philox; init!(sys, :up / :down). */
MCX_API mcx_status mcx_graph_init_random(mcx_graph* g, uint64_t seed, uint32_t stream);
MCX_API mcx_status mcx_graph_init_uniform(mcx_graph* g, int8_t value);
/* energy(sys; full) and magnetization(sys; full) (ising.jl:17-18): the cached values,
 * or with full != 0 a recompute from the spins (_full_energy, ising.jl:185, :349) that
 * also resets the cache (_recompute_cached!).  Waits for the stream. */
MCX_API mcx_status mcx_graph_energy(mcx_graph* g, int full, double* energy,
                                    int64_t* magnetization);
/* delta_energy(sys, i) (ising.jl:20-23, :198, :362) for 0-based site i; waits. */
MCX_API mcx_status mcx_graph_delta_energy(mcx_graph* g, int64_t i, double* delta_energy);
/* modify!(sys, i, Δpair, Δspin) (SpinSystems/src/ising.jl:200-218, :364-377) with the
 * flip_changes of site i (:187-192, :351-356): flips spin i and updates the cached energy and
 * magnetization. */
MCX_API mcx_status mcx_graph_flip(mcx_graph* g, int64_t i);
/* delta_energy(sys, i, s_new) (SpinSystems/src/blume_capel.jl:36-39; for an Ising graph s_new = -s_i is
 * the flip and s_new = s_i gives 0) and modify! to s_new with propose_changes
 * (:235-241, :250-272, :423-429, :438-460). */
MCX_API mcx_status mcx_graph_delta_energy_to(mcx_graph* g, int64_t i, int8_t s_new,
                                             double* delta_energy);
MCX_API mcx_status mcx_graph_set_site(mcx_graph* g, int64_t i, int8_t s_new);
/* `nsweeps` sweeps of n spin_flip!(sys, alg) each (ising.jl:25-58 with accept!,
 * src/algorithms/metropolis.jl:14-17, :121-127, importance_sampling.jl:80-85): the
 * reference's FP64 decisions -- Metropolis lr = -beta*ΔE, accept if lr > 0 or
 * u < exp(lr); Glauber u < logistic(lr); HeatBath s = u < logistic(beta*s*ΔE) ? +1 : -1
 * -- with exp the library's own (bit-identical on host and device) and u a 53-bit
 * uniform: the l-th site of colour class c takes words 2b, 2b+1 (b = (l>>5)&1) of the
 * Philox block (B, sweep lo, sweep hi16 | 7<<24, stream), B = B_c + 32 (l>>6) + (l&31),
 * B_c the sum of 32 ceil(n_c'/64) over the earlier classes.
 *   E_series: host float64[nsweeps] of the cached energy after each sweep, or NULL.
 *   M_series: host int64[nsweeps] of the magnetization after each sweep, or NULL.
 *   counters: accumulated (HeatBath: accepted = spins that changed), or NULL. */
MCX_API mcx_status mcx_graph_sweep(mcx_graph* g, mcx_algorithm alg, double beta, mcx_rng* rng,
                                   int64_t nsweeps, double* E_series, int64_t* M_series,
                                   mcx_counters* counters);

/* `nattempts` x spin_flip!(sys, alg) in the reference's own order on a general graph: a
 * uniformly random vertex per attempt (pick_site, SpinSystems/src/abstractions.jl:19) and the
 * site's FP64 rule of mcx_graph_sweep (Ising: ising.jl:25-58; Blume-Capel:
 * SpinSystems/src/blume_capel.jl:41-85).  Attempt a = rng->counter + k draws
 * Philox4x32-10(seed, (a lo, a hi, 5<<24, stream)): vertex ((w0<<32)|w1) mod n, u = u53(w2, w3);
 * Blume-Capel Metropolis / Glauber proposals take the top bit of word 0 of (a lo, a hi, 6<<24,
 * stream).  rng->counter advances by nattempts.  Serial (one thread applies the attempts in
 * order); the cached energy is the sequential FP64 sum of the accepted changes.  counters may
 * be NULL (the call then only enqueues work). */
MCX_API mcx_status mcx_graph_spin_flip(mcx_graph* g, mcx_algorithm alg, double beta, mcx_rng* rng,
                                       int64_t nattempts, mcx_counters* counters);

/* ---------------------------------------------------------- measurements -- */
/* integrated_autocorrelation_times(traces; min_points, max_lag, c)
 * (src/measurements/autocorrelations.jl:28-110) on the device, for traces in host
 * memory: trace k is values[offsets[k] .. offsets[k+1]) (float64).  tau = 1/2 + sum of
 * the normalised autocovariances C(t), t = 1, 2, ..., stopping at the first C(t) <= 0
 * or when t > c * tau; at least 0.5 (0.5 for a constant trace).  Lag window
 * min(max_lag, floor(n/2)) (max_lag <= 0: floor(n/2)); traces with fewer than
 * min_points samples or an empty window give NaN.  c <= 0 or min_points < 2:
 * MCX_ERR_INVALID_ARG.  Waits for the stream. */
MCX_API mcx_status mcx_tau_int(mcx_ctx* ctx, const double* values, const int64_t* offsets,
                               int32_t ntraces, int64_t min_points, int64_t max_lag, double c,
                               double* taus);
/* tau_int of the per-sweep series of the last mcx_sweep (lattice) or mcx_graph_sweep
 * (graph) call, read where it lies on the device: quantity 0 energy, 1 magnetization.
 * The single-trace rules: at least 2 sweeps, max_lag <= floor(n/2) (<= 0: floor(n/2)),
 * else MCX_ERR_INVALID_ARG. */
MCX_API mcx_status mcx_lattice_tau_int(mcx_lattice* lat, int quantity, int64_t max_lag, double c,
                                       double* tau);
MCX_API mcx_status mcx_graph_tau_int(mcx_graph* g, int quantity, int64_t max_lag, double c,
                                     double* tau);

/* ----------------------------------------------------------- no allocation -- */
/* mcx_sweep_noalloc has no counterpart in the reference.  It runs the same sweeps as
 * mcx_sweep for callers that must not have device memory allocated during the call:
 * programs whose GPU memory all belongs to another allocator (CUDA.jl's pool in Julia,
 * PyTorch's caching allocator) or a service that reserved its HBM up front.  For them
 * a library-side cudaMalloc bypasses the owner's accounting and can fail at run time,
 * and cudaFree waits for the whole device.  This call uses no cudaMalloc, cudaFree or
 * other allocating routine: its scratch (the per-sweep partial sums and the accepted
 * counter) is one fixed device array of MCX_NOALLOC_MAX_SWEEPS sweeps (96 KiB) that
 * every GPU which loads the library holds until the process exits; a call with more
 * sweeps returns MCX_ERR_INVALID_ARG.  int8 lattices only.
 *   obs_series_dev: caller-owned device int64[nsweeps*3], written with the per-sweep
 *                   (pair_sum, spin_sum, spin2_sum), or NULL.
 *   accepted_dev:   caller-owned device uint64, set to this call's accepted moves, or NULL.
 * The call only enqueues work on the context stream; the lattice's cached bookkeeping
 * (mcx_observables) is updated.  The series the library keeps for the lattice is not
 * written: after this call mcx_read_series and mcx_lattice_tau_int find no recorded
 * sweeps (MCX_ERR_INVALID_ARG) until the next mcx_sweep.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) and keeps it for the life
 * of the process; make that first call before any stream capture, and do not use the
 * library on a device after resetting it (cudaDeviceReset).  Every call shares the
 * array and clears the part it uses; calls whose work overlaps on the GPU (other
 * streams or contexts on the same device) race on it and must be serialized by the
 * caller. */
#define MCX_NOALLOC_MAX_SWEEPS 4096
MCX_API mcx_status mcx_sweep_noalloc(mcx_lattice* lat, mcx_algorithm alg, double beta,
                                     mcx_rng* rng, int64_t nsweeps, int64_t* obs_series_dev,
                                     uint64_t* accepted_dev);

#ifdef __cplusplus
}
#endif
#endif /* MCX_H */

// mcx_serve.cu -- serving: continuous batching of simulation jobs of mixed size.
//
// Jobs (a canonical sweep run or a Multicanonical run on a 2-D Ising / Blume-Capel
// lattice) are queued by mcx_server_submit.  Every mcx_server_step is one
// scheduling iteration:
//   1. admit queued jobs in arrival order while the server's HBM budget and job slots
//      allow (lattice, per-sweep series and histograms are allocated on the device
//      and stay there until the job retires);
//   2. advance every active job by up to `chunk` sweeps: for each sweep of the chunk
//      one launch per colour covers the tiles of all active canonical jobs (jobs of
//      every size and model in the same launch), and one flat-histogram launch covers
//      all active Multicanonical jobs;
//   3. retire the jobs that finished: results to the caller's host buffers, device
//      memory freed, so queued jobs can be admitted at the next step.
// A job's random stream is its own (seed, stream) and the per-sweep counter, so its
// result does not depend on which other jobs share the device: identical alone and
// in the mix.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <thread>
#include <vector>

#include "mcx_cb.cuh"
#include "mcx_device.cuh"
#include "mcx_flathist.cuh"
#include "mcx_internal.h"
#include "mcx_sweep.cuh"

namespace mcx {

struct SrvJobDev {
    int8_t* col[2];
    long long* series;  // this iteration's first sweep row of the per-sweep deltas
    unsigned long long* acc;
    int W, Ly, rows, cpr, V, model, hb, todo;
    uint32_t k0, k1, stream, m_cpr;
    unsigned long long t0;
};

struct SrvTile {
    int job, c_begin, c_end, pad;
};

__device__ __forceinline__ uint32_t sdiv(uint32_t n, uint32_t m) { return m ? __umulhi(n, m) : n; }

template <int V, int MODEL, bool HB>
__device__ __forceinline__ void srv_tile(const SrvJobDev& J, const SrvTile& tl, int colour, unsigned long long t,
                                         const unsigned long long* s_thr, int& nacc, int& a1, int& a2, int& a3) {
    constexpr int Z = 4;
    constexpr int NW = V / 4;
    int8_t* cur = J.col[colour];
    const int8_t* oth = J.col[1 - colour];
    const uint32_t w2a = ctr_word2(t, colour, P_ACCEPT), w2p = ctr_word2(t, colour, P_PROPOSE);
    for (int g = tl.c_begin + (int)threadIdx.x; g < tl.c_end; g += blockDim.x) {
        const int r = (int)sdiv((uint32_t)g, J.m_cpr);
        const int q = g - r * J.cpr;
        const RowInfo ri = row_info_yz(r, 0, J.Ly, 1, colour, 2);
        Chunk<2, V> ch;
        ch.load(cur, oth, J.W, r, q * V, ri);
        const uint32_t c0 = (uint32_t)(((unsigned long long)r * J.W + q * V) >> 2);
        BcLanes ln;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            uint32_t nbw[Z];
#pragma unroll
            for (int d = 0; d < Z; ++d) nbw[d] = ch.nb[d][w];
            const uint4 ra = philox10(make_uint4(c0 + w, (uint32_t)t, w2a, J.stream), J.k0, J.k1);
            if (MODEL == 0) {
                const uint32_t fb = ising_word<Z, HB>(nbw, ch.own[w], ra, s_thr, nacc, a1, a2);
                ch.own[w] ^= fb * 0xFEu;
            } else {
                uint4 rp = make_uint4(0, 0, 0, 0);
                if (!HB) rp = philox10(make_uint4(c0 + w, (uint32_t)t, w2p, J.stream), J.k0, J.k1);
                ch.own[w] = bc_word_swar<Z, HB>(nbw, ch.own[w], ra, rp, s_thr, nacc, ln);
            }
        }
        if (MODEL != 0) bc_lanes_fold<Z>(ln, a1, a2, a3);
        store_row<V>(cur + (long long)r * J.W + q * V, ch.own);
    }
}

// One colour of sweep s of the current chunk, for the tiles of every active
// canonical job (tiles of jobs with fewer than s+1 sweeps left are skipped).
__global__ void __launch_bounds__(256) k_srv_half(const SrvJobDev* jobs, const SrvTile* tiles, int ntiles,
                                                  const unsigned long long* tables, int colour, int s) {
    __shared__ __align__(16) unsigned long long s_thr[kMaxTable];
    for (int ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
        const SrvTile tl = tiles[ti];
        const SrvJobDev J = jobs[tl.job];
        if (s >= J.todo) continue;  // uniform over the block
        __syncthreads();
        for (int i = threadIdx.x; i < kMaxTable; i += blockDim.x) {
            const unsigned long long x = tables[(size_t)tl.job * kMaxTable + i];
            s_thr[i] = J.model == 0 ? ising_tab_entry(x, i, 4, J.hb != 0) : x;
        }
        __syncthreads();
        const unsigned long long t = J.t0 + (unsigned long long)s;
        int nacc = 0, a1 = 0, a2 = 0, a3 = 0;
        const int key = J.V * 4 + J.model * 2 + J.hb;
        switch (key) {
            case 16 * 4 + 0: srv_tile<16, 0, false>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            case 16 * 4 + 1: srv_tile<16, 0, true>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            case 16 * 4 + 2: srv_tile<16, 1, false>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            case 16 * 4 + 3: srv_tile<16, 1, true>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            case 8 * 4 + 0: srv_tile<8, 0, false>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            case 8 * 4 + 1: srv_tile<8, 0, true>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            case 8 * 4 + 2: srv_tile<8, 1, false>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            case 8 * 4 + 3: srv_tile<8, 1, true>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            case 4 * 4 + 0: srv_tile<4, 0, false>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            case 4 * 4 + 1: srv_tile<4, 0, true>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            case 4 * 4 + 2: srv_tile<4, 1, false>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
            default: srv_tile<4, 1, true>(J, tl, colour, t, s_thr, nacc, a1, a2, a3); break;
        }
        long long dP, dM, dQ;
        if (J.model == 0) {
            ising_deltas<4>(nacc, a1, a2, dP, dM);
            dQ = 0;
        } else {
            dP = a1;
            dM = a2;
            dQ = a3;
        }
        long long v[4] = {dP, dM, dQ, (long long)nacc};
        unsigned long long* const dst[4] = {(unsigned long long*)&J.series[3 * s],
                                            (unsigned long long*)&J.series[3 * s + 1],
                                            (unsigned long long*)&J.series[3 * s + 2], J.acc};
        block_add_atomic<4>(v, dst);
    }
}

}  // namespace mcx

using namespace mcx;

namespace {

enum JobState { JOB_PENDING = 0, JOB_ACTIVE = 1, JOB_DONE = 2, JOB_CANCELLED = 3, JOB_FAILED = 4 };

struct SrvJob {
    uint64_t id = 0;
    mcx_job spec{};
    std::vector<double> lnw0;
    mcx_lattice* lat = nullptr;
    mcx_flathist* fh = nullptr;
    int64_t done = 0;
    long long P = 0, M = 0, Q = 0;
    uint64_t steps = 0, accepted = 0;
    double t_submit = 0, t_admit = 0, t_finish = 0;
    int state = JOB_PENDING;
    mcx_status status = MCX_OK;
    uint64_t bytes = 0;
    Table table{};
    int inflight = 0;       // sweeps of the Multicanonical launch in flight (0: none)
    bool cancel_req = false;
};

double now_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct mcx_server {
    mcx_ctx* ctx = nullptr;
    mcx::CtxHold hold;  // keeps ctx alive while this object exists
    uint64_t budget = 0, used = 0, peak = 0;
    int max_jobs = 0, chunk = 0;
    uint64_t next_id = 1;
    std::map<uint64_t, SrvJob*> jobs;
    std::deque<SrvJob*> pending;
    std::vector<SrvJob*> active;
    std::chrono::steady_clock::time_point t0;
    // device descriptors, grown as needed
    SrvJobDev* d_jobs = nullptr;
    size_t cap_jobs = 0;
    SrvTile* d_tiles = nullptr;
    size_t cap_tiles = 0;
    unsigned long long* d_tables = nullptr;
    size_t cap_tables = 0;
    FHWalker* d_walkers = nullptr;
    size_t cap_walkers = 0;
    uint64_t iterations = 0, jobs_done = 0, attempts_done = 0;
    // Multicanonical jobs run on their own stream, one launch in flight at a time, so
    // that canonical jobs never wait for the (serial, long) walker chains
    cudaStream_t mstream = nullptr;
    cudaEvent_t mdone = nullptr;
    bool minflight = false;
    std::vector<FHWalker> mwalk;
    std::vector<SrvJob*> mjobs;
    std::vector<SrvJob*> deferred;  // finished jobs whose memory is freed when no walker launch runs
};

namespace {

template <typename T>
mcx_status grow(mcx_server* s, T** p, size_t* cap, size_t n) {
    if (n <= *cap) return MCX_OK;
    size_t c = *cap ? *cap : 16;
    while (c < n) c *= 2;
    void* q = nullptr;
    MCX_CHECK(dev_alloc(s->ctx, &q, c * sizeof(T)));
    dev_free(s->ctx, *p, *cap * sizeof(T));
    *p = (T*)q;
    *cap = c;
    return MCX_OK;
}

int64_t lattice_bytes(const mcx_job& j) {
    const int64_t N = (int64_t)j.L[0] * j.L[1];
    int64_t cap = 64;
    while (cap < j.nsweeps) cap *= 2;
    return 2 * N + 32 + cap * 24;  // colours + staging, state + counter, series
}

uint64_t job_bytes(const mcx_job& j) {
    uint64_t b = (uint64_t)lattice_bytes(j);
    if (j.kind == MCX_JOB_MULTICANONICAL) b += (uint64_t)j.nbins * 17 + 24;
    return b;
}

mcx_status validate(const mcx_job& j) {
    if (j.model != MCX_ISING && j.model != MCX_BLUME_CAPEL) return fail(MCX_ERR_INVALID_ARG, "job: unknown model");
    if (j.dim != 2) return fail(MCX_ERR_INVALID_ARG, "job: the serving loop runs 2-D lattices");
    for (int d = 0; d < 2; ++d)
        if (j.L[d] < 8 || j.L[d] % 8) return fail(MCX_ERR_INVALID_ARG, "job: sides must be multiples of 8");
    if (j.nsweeps < 1) return fail(MCX_ERR_INVALID_ARG, "job: nsweeps >= 1");
    if (j.kind != MCX_JOB_CANONICAL && j.kind != MCX_JOB_MULTICANONICAL)
        return fail(MCX_ERR_INVALID_ARG, "job: unknown kind");
    if (!std::isfinite(j.beta) || !std::isfinite(j.J) || !std::isfinite(j.D) || !std::isfinite(j.h))
        return fail(MCX_ERR_INVALID_ARG, "job: non-finite parameter");
    if (j.kind == MCX_JOB_CANONICAL && j.alg != MCX_METROPOLIS && j.alg != MCX_GLAUBER && j.alg != MCX_HEATBATH)
        return fail(MCX_ERR_INVALID_ARG, "job: unknown algorithm");
    if (j.kind == MCX_JOB_MULTICANONICAL) {
        if (j.nbins < 1 || j.bin_step < 1) return fail(MCX_ERR_INVALID_ARG, "job: bad bins");
        if ((double)(long long)j.J != j.J || (double)(long long)j.D != j.D || (double)(long long)j.h != j.h)
            return fail(MCX_ERR_INVALID_ARG, "job: Multicanonical jobs need integer J, D, h");
        if (!fh_window_ok(2, (long long)j.J, (long long)j.D, (long long)j.h, j.bin_step))
            return fail(MCX_ERR_INVALID_ARG, "job: one move may change the energy by more than the ln g window holds");
    }
    return MCX_OK;
}

void release(mcx_server* s, SrvJob* j) {
    if (j->lat) mcx_lattice_destroy(j->lat);
    if (j->fh) mcx_flathist_destroy(j->fh);
    j->lat = nullptr;
    j->fh = nullptr;
    s->used -= j->bytes;
}

mcx_status admit(mcx_server* s, SrvJob* j) {
    const mcx_job& sp = j->spec;
    const int32_t L[3] = {sp.L[0], sp.L[1], 1};
    MCX_CHECK(mcx_lattice_create(s->ctx, (mcx_model)sp.model, 2, L, MCX_LAYOUT_INT8, sp.J, sp.D, sp.h, &j->lat));
    s->used += j->bytes;
    s->peak = std::max(s->peak, s->used);
    MCX_CHECK(mcx_init_random(j->lat, sp.seed, sp.stream));
    MCX_CHECK(ensure_series(j->lat, sp.nsweeps));
    MCX_CUDA(cudaMemsetAsync(j->lat->d_series, 0, (size_t)sp.nsweeps * 24, s->ctx->stream));
    MCX_CUDA(cudaMemsetAsync(j->lat->d_acc, 0, 8, s->ctx->stream));
    if (sp.kind == MCX_JOB_CANONICAL) {
        MCX_CHECK(build_table(j->lat, (mcx_algorithm)sp.alg, sp.beta, &j->table));
    } else {
        MCX_CHECK(mcx_flathist_create(s->ctx, sp.bin_start, sp.bin_step, sp.nbins, &j->fh));
        if (!j->lnw0.empty())
            MCX_CUDA(cudaMemcpyAsync(j->fh->d_lnw, j->lnw0.data(), j->lnw0.size() * 8, cudaMemcpyHostToDevice,
                                     s->ctx->stream));
        long long st[3];
        MCX_CUDA(cudaMemcpyAsync(st, j->lat->d_state, 24, cudaMemcpyDeviceToHost, s->ctx->stream));
        MCX_CUDA(cudaStreamSynchronize(s->ctx->stream));
        j->P = st[0];
        j->M = st[1];
        j->Q = st[2];
    }
    j->state = JOB_ACTIVE;
    j->t_admit = now_s(s->t0);
    return MCX_OK;
}

mcx_status finish(mcx_server* s, SrvJob* j) {
    const mcx_job& sp = j->spec;
    mcx_ctx* ctx = s->ctx;
    if (sp.kind == MCX_JOB_CANONICAL) {
        MCX_CHECK(finish_series(j->lat, sp.nsweeps));
        unsigned long long acc = 0;
        long long st[3];
        MCX_CUDA(cudaMemcpyAsync(&acc, j->lat->d_acc, 8, cudaMemcpyDeviceToHost, ctx->stream));
        MCX_CUDA(cudaMemcpyAsync(st, j->lat->d_state, 24, cudaMemcpyDeviceToHost, ctx->stream));
        if (sp.obs_series)
            MCX_CUDA(cudaMemcpyAsync(sp.obs_series, j->lat->d_series, (size_t)sp.nsweeps * 24, cudaMemcpyDeviceToHost,
                                     ctx->stream));
        MCX_CUDA(cudaStreamSynchronize(ctx->stream));
        j->P = st[0];
        j->M = st[1];
        j->Q = st[2];
        j->steps = (uint64_t)j->lat->N * (uint64_t)sp.nsweeps;
        j->accepted = acc;
    } else {
        if (sp.obs_series)
            MCX_CUDA(cudaMemcpyAsync(sp.obs_series, j->lat->d_series, (size_t)sp.nsweeps * 24, cudaMemcpyDeviceToHost,
                                     ctx->stream));
        if (sp.histogram)
            MCX_CUDA(cudaMemcpyAsync(sp.histogram, j->fh->d_H, (size_t)sp.nbins * 8, cudaMemcpyDeviceToHost, ctx->stream));
        if (sp.logweight_out)
            MCX_CUDA(cudaMemcpyAsync(sp.logweight_out, j->fh->d_lnw, (size_t)sp.nbins * 8, cudaMemcpyDeviceToHost,
                                     ctx->stream));
        MCX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    if (sp.final_spins) MCX_CHECK(mcx_get_spins(j->lat, sp.final_spins, (size_t)j->lat->N));
    j->t_finish = now_s(s->t0);
    j->state = j->status == MCX_OK ? JOB_DONE : JOB_FAILED;
    s->jobs_done += 1;
    s->attempts_done += j->steps;
    // freeing synchronises the device, which would wait for a walker launch in flight
    if (s->minflight) s->deferred.push_back(j);
    else release(s, j);
    return MCX_OK;
}

// Results of the walker launch in flight, when it has completed: job bookkeeping,
// completion of finished (or cancelled) jobs.  Returns MCX_OK while it still runs.
mcx_status collect_muca(mcx_server* s) {
    if (!s->minflight) return MCX_OK;
    const cudaError_t q = cudaEventQuery(s->mdone);
    if (q == cudaErrorNotReady) return MCX_OK;
    if (q != cudaSuccess) return cuda_fail(q, "walker launch");
    MCX_CUDA(cudaMemcpy(s->mwalk.data(), s->d_walkers, s->mwalk.size() * sizeof(FHWalker), cudaMemcpyDeviceToHost));
    s->minflight = false;
    for (size_t i = 0; i < s->mjobs.size(); ++i) {
        SrvJob* j = s->mjobs[i];
        const FHWalker& w = s->mwalk[i];
        j->P = w.P;
        j->M = w.M;
        j->Q = w.Q;
        j->steps += w.steps;
        j->accepted += w.accepted;
        j->done += j->inflight;
        j->inflight = 0;
        if (w.status) {
            j->status = MCX_ERR_OUT_OF_RANGE;
            j->done = j->spec.nsweeps;  // stops here, like the reference's BoundsError
        }
        long long st[3] = {j->P, j->M, j->Q};
        MCX_CUDA(cudaMemcpy(j->lat->d_state, st, 24, cudaMemcpyHostToDevice));
    }
    std::vector<SrvJob*> still;
    for (SrvJob* j : s->active) {
        if (j->spec.kind == MCX_JOB_CANONICAL) {
            still.push_back(j);
        } else if (j->cancel_req) {
            j->state = JOB_CANCELLED;
            j->t_finish = now_s(s->t0);
            release(s, j);
        } else if (j->done >= j->spec.nsweeps) {
            MCX_CHECK(finish(s, j));
        } else {
            still.push_back(j);
        }
    }
    s->active.swap(still);
    s->mjobs.clear();
    return MCX_OK;
}

// Starts one walker launch (chunk sweeps) for every active Multicanonical job.
mcx_status launch_muca(mcx_server* s) {
    if (s->minflight) return MCX_OK;
    s->mwalk.clear();
    s->mjobs.clear();
    for (SrvJob* j : s->active) {
        if (j->spec.kind != MCX_JOB_MULTICANONICAL || j->done >= j->spec.nsweeps) continue;
        const int todo = (int)std::min<int64_t>(s->chunk, j->spec.nsweeps - j->done);
        const mcx_lattice* L = j->lat;
        FHWalker w;
        std::memset(&w, 0, sizeof(w));
        w.g.W = (int)L->W;
        w.g.Ly = (int)L->L[1];
        w.g.Lz = 1;
        w.g.dim = 2;
        w.g.model = L->model == MCX_ISING ? 0 : 1;
        w.g.J = (long long)L->J;
        w.g.D = (long long)L->D;
        w.g.h = (long long)L->h;
        w.g.start = j->spec.bin_start;
        w.g.step = j->spec.bin_step;
        w.g.nbins = j->spec.nbins;
        w.g.shift = fh_shift(j->spec.bin_step);
        w.g.mode = 0;
        w.g.nsweeps = todo;
        w.col[0] = L->d_col[0];
        w.col[1] = L->d_col[1];
        w.lnw = j->fh->d_lnw;
        w.H = j->fh->d_H;
        w.series = (long long*)L->d_series + 3 * j->done;
        w.P = j->P;
        w.M = j->M;
        w.Q = j->Q;
        w.sweep0 = (unsigned long long)j->done;
        w.k0 = (uint32_t)j->spec.seed;
        w.k1 = (uint32_t)(j->spec.seed >> 32);
        w.stream = j->spec.stream;
        j->inflight = todo;
        s->mwalk.push_back(w);
        s->mjobs.push_back(j);
    }
    if (s->mjobs.empty()) return MCX_OK;
    if (!s->mstream) {
        MCX_CUDA(cudaStreamCreateWithFlags(&s->mstream, cudaStreamNonBlocking));
        MCX_CUDA(cudaEventCreateWithFlags(&s->mdone, cudaEventDisableTiming));
    }
    // the walkers' lattices were initialised on the context stream
    MCX_CUDA(cudaStreamSynchronize(s->ctx->stream));
    MCX_CHECK(grow(s, &s->d_walkers, &s->cap_walkers, s->mwalk.size()));
    MCX_CUDA(cudaMemcpyAsync(s->d_walkers, s->mwalk.data(), s->mwalk.size() * sizeof(FHWalker), cudaMemcpyHostToDevice,
                             s->mstream));
    MCX_CHECK(launch_flathist_on(s->ctx, s->mstream, s->d_walkers, (int)s->mwalk.size()));
    MCX_CUDA(cudaEventRecord(s->mdone, s->mstream));
    s->minflight = true;
    return MCX_OK;
}

// one scheduling iteration
mcx_status step(mcx_server* s) {
    mcx_ctx* ctx = s->ctx;
    // 1. admission in arrival order, by slots and HBM budget
    while (!s->pending.empty() && (int)s->active.size() < s->max_jobs) {
        SrvJob* j = s->pending.front();
        if (s->budget && s->used + j->bytes > s->budget) break;
        s->pending.pop_front();
        mcx_status st = admit(s, j);
        if (st != MCX_OK) {
            j->status = st;
            j->state = JOB_FAILED;
            j->t_finish = now_s(s->t0);
            release(s, j);
            continue;
        }
        s->active.push_back(j);
    }
    // 2. Multicanonical jobs: collect a completed walker launch, free deferred memory
    //    while nothing runs on the walker stream, start the next launch
    MCX_CHECK(collect_muca(s));
    if (!s->minflight) {
        for (SrvJob* j : s->deferred) release(s, j);
        s->deferred.clear();
    }
    MCX_CHECK(launch_muca(s));
    // 3. one chunk for every active canonical job
    std::vector<SrvJobDev> jd;
    std::vector<SrvTile> tiles;
    std::vector<unsigned long long> tabs;
    std::vector<SrvJob*> canon;
    int chunk = 0;
    for (SrvJob* j : s->active) {
        if (j->spec.kind != MCX_JOB_CANONICAL) continue;
        const int todo = (int)std::min<int64_t>(s->chunk, j->spec.nsweeps - j->done);
        chunk = std::max(chunk, todo);
        const mcx_lattice* L = j->lat;
        SrvJobDev d;
        std::memset(&d, 0, sizeof(d));
        d.col[0] = L->d_col[0];
        d.col[1] = L->d_col[1];
        d.series = (long long*)L->d_series + 3 * j->done;
        d.acc = L->d_acc;
        d.W = (int)L->W;
        d.Ly = (int)L->L[1];
        d.rows = (int)L->rows;
        d.V = L->W % 16 == 0 ? 16 : (L->W % 8 == 0 ? 8 : 4);
        d.cpr = d.W / d.V;
        d.model = L->model == MCX_ISING ? 0 : 1;
        d.hb = j->spec.alg == MCX_HEATBATH;
        d.todo = todo;
        d.k0 = (uint32_t)j->spec.seed;
        d.k1 = (uint32_t)(j->spec.seed >> 32);
        d.stream = j->spec.stream;
        d.m_cpr = d.cpr <= 1 ? 0u : (uint32_t)(((1ull << 32) + d.cpr - 1) / d.cpr);
        d.t0 = (unsigned long long)j->done;
        const int idx = (int)jd.size();
        jd.push_back(d);
        for (int i = 0; i < kMaxTable; ++i) tabs.push_back(i < j->table.n ? j->table.thr[i] : 0ull);
        const int nch = d.cpr * d.rows, per = 256 * (16 / d.V);
        for (int c = 0; c < nch; c += per) tiles.push_back(SrvTile{idx, c, std::min(nch, c + per), 0});
        canon.push_back(j);
    }
    if (canon.empty()) {
        if (s->minflight) std::this_thread::sleep_for(std::chrono::microseconds(50));  // walkers only: do not spin
        return MCX_OK;
    }
    MCX_CHECK(grow(s, &s->d_jobs, &s->cap_jobs, jd.size()));
    MCX_CHECK(grow(s, &s->d_tiles, &s->cap_tiles, tiles.size()));
    MCX_CHECK(grow(s, &s->d_tables, &s->cap_tables, tabs.size()));
    MCX_CUDA(cudaMemcpyAsync(s->d_jobs, jd.data(), jd.size() * sizeof(SrvJobDev), cudaMemcpyHostToDevice, ctx->stream));
    MCX_CUDA(cudaMemcpyAsync(s->d_tiles, tiles.data(), tiles.size() * sizeof(SrvTile), cudaMemcpyHostToDevice,
                             ctx->stream));
    MCX_CUDA(cudaMemcpyAsync(s->d_tables, tabs.data(), tabs.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
    const int grid = occupancy_grid(ctx, (const void*)k_srv_half, (long long)tiles.size() * 256, 256, 0);
    for (int sw = 0; sw < chunk; ++sw)
        for (int c = 0; c < 2; ++c)
            k_srv_half<<<grid, 256, 0, ctx->stream>>>(s->d_jobs, s->d_tiles, (int)tiles.size(), s->d_tables, c, sw);
    count_launch(ctx, 2 * (uint64_t)chunk);
    MCX_CUDA(cudaGetLastError());
    MCX_CUDA(cudaStreamSynchronize(ctx->stream));
    s->iterations += 1;
    // 4. progress and retirement of the canonical jobs
    std::vector<SrvJob*> still;
    for (SrvJob* j : s->active) {
        if (j->spec.kind == MCX_JOB_CANONICAL) {
            j->done += std::min<int64_t>(s->chunk, j->spec.nsweeps - j->done);
            if (j->done >= j->spec.nsweeps) {
                MCX_CHECK(finish(s, j));
                continue;
            }
        }
        still.push_back(j);
    }
    s->active.swap(still);
    return MCX_OK;
}

}  // namespace

extern "C" {

MCX_API mcx_status mcx_server_create(mcx_ctx* ctx, uint64_t hbm_budget, int32_t max_jobs, int32_t chunk_sweeps,
                                     mcx_server** out) {
    if (!ctx || !out) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (max_jobs < 1 || chunk_sweeps < 1) return fail(MCX_ERR_INVALID_ARG, "max_jobs and chunk_sweeps must be >= 1");
    mcx_server* s = new mcx_server();
    s->ctx = ctx;
    s->hold.set(ctx);
    s->budget = hbm_budget;
    s->max_jobs = max_jobs;
    s->chunk = chunk_sweeps;
    s->t0 = std::chrono::steady_clock::now();
    *out = s;
    return MCX_OK;
}

MCX_API mcx_status mcx_server_destroy(mcx_server* s) {
    if (!s) return MCX_OK;
    cudaStreamSynchronize(s->ctx->stream);
    if (s->mstream) cudaStreamSynchronize(s->mstream);
    s->minflight = false;
    for (auto& kv : s->jobs) {
        if (kv.second->lat || kv.second->fh) release(s, kv.second);
        delete kv.second;
    }
    dev_free(s->ctx, s->d_jobs, s->cap_jobs * sizeof(SrvJobDev));
    dev_free(s->ctx, s->d_tiles, s->cap_tiles * sizeof(SrvTile));
    dev_free(s->ctx, s->d_tables, s->cap_tables * 8);
    dev_free(s->ctx, s->d_walkers, s->cap_walkers * sizeof(FHWalker));
    if (s->mdone) cudaEventDestroy(s->mdone);
    if (s->mstream) cudaStreamDestroy(s->mstream);
    delete s;
    return MCX_OK;
}

MCX_API mcx_status mcx_server_submit(mcx_server* s, const mcx_job* job, uint64_t* job_id) {
    if (!s || !job || !job_id) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    MCX_CHECK(validate(*job));
    const uint64_t bytes = job_bytes(*job);
    if (s->budget && bytes > s->budget)
        return fail(MCX_ERR_BUDGET, "job needs %llu bytes, more than the server budget %llu",
                    (unsigned long long)bytes, (unsigned long long)s->budget);
    SrvJob* j = new SrvJob();
    j->id = s->next_id++;
    j->spec = *job;
    j->bytes = bytes;
    if (job->kind == MCX_JOB_MULTICANONICAL && job->logweight)
        j->lnw0.assign(job->logweight, job->logweight + job->nbins);
    j->spec.logweight = nullptr;
    j->t_submit = now_s(s->t0);
    s->jobs[j->id] = j;
    s->pending.push_back(j);
    *job_id = j->id;
    return MCX_OK;
}

MCX_API mcx_status mcx_server_step(mcx_server* s, int32_t* active, int32_t* pending) {
    if (!s) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    MCX_CHECK(step(s));
    if (active) *active = (int32_t)s->active.size();
    if (pending) *pending = (int32_t)s->pending.size();
    return MCX_OK;
}

MCX_API mcx_status mcx_server_poll(mcx_server* s, uint64_t job_id, mcx_job_result* res) {
    if (!s || !res) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return fail(MCX_ERR_NOT_FOUND, "unknown job %llu", (unsigned long long)job_id);
    const SrvJob* j = it->second;
    std::memset(res, 0, sizeof(*res));
    res->state = j->state;
    res->status = j->status;
    res->pair_sum = j->P;
    res->spin_sum = j->M;
    res->spin2_sum = j->Q;
    res->attempts = j->steps;
    res->accepted = j->accepted;
    res->submit_s = j->t_submit;
    res->admit_s = j->t_admit;
    res->finish_s = j->t_finish;
    res->sweeps_done = j->done;
    if (j->state == JOB_PENDING || j->state == JOB_ACTIVE) return MCX_ERR_NOT_READY;
    return MCX_OK;
}

MCX_API mcx_status mcx_server_cancel(mcx_server* s, uint64_t job_id) {
    if (!s) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end()) return fail(MCX_ERR_NOT_FOUND, "unknown job %llu", (unsigned long long)job_id);
    SrvJob* j = it->second;
    if (j->state == JOB_PENDING) {
        s->pending.erase(std::find(s->pending.begin(), s->pending.end(), j));
    } else if (j->state == JOB_ACTIVE) {
        if (j->inflight) {  // its walker launch is running: cancelled when it completes
            j->cancel_req = true;
            return MCX_OK;
        }
        MCX_CUDA(cudaStreamSynchronize(s->ctx->stream));
        s->active.erase(std::find(s->active.begin(), s->active.end(), j));
        if (s->minflight) s->deferred.push_back(j);
        else release(s, j);
    } else {
        return MCX_OK;
    }
    j->state = JOB_CANCELLED;
    j->t_finish = now_s(s->t0);
    return MCX_OK;
}

MCX_API mcx_status mcx_server_get_stats(mcx_server* s, mcx_server_stats* st) {
    if (!s || !st) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    std::memset(st, 0, sizeof(*st));
    st->active = (int32_t)s->active.size();
    st->pending = (int32_t)s->pending.size();
    st->iterations = s->iterations;
    st->jobs_done = s->jobs_done;
    st->attempts_done = s->attempts_done;
    st->bytes_in_use = s->used;
    st->peak_bytes = s->peak;
    st->now_s = now_s(s->t0);
    return MCX_OK;
}

}  // extern "C"

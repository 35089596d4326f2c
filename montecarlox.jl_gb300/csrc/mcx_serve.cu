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
#include <atomic>
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
                uint32_t bits = 0;
                if (!HB) bits = bc_site_bits(philox10(make_uint4(c0 + w, (uint32_t)t, w2p, J.stream), J.k0, J.k1));
                ch.own[w] = bc_word_swar<Z, HB>(nbw, ch.own[w], ra, bits, s_thr, nacc, ln);
            }
        }
        if (MODEL != 0) bc_lanes_fold<Z>(ln, a1, a2, a3);
        store_row<V>(cur + (long long)r * J.W + q * V, ch.own);
    }
}

// One colour of sweep s of the current chunk, for the tiles of every active
// canonical job (tiles of jobs with fewer than s+1 sweeps left are skipped).  Every block
// takes an equal contiguous range of the tiles (laid out job by job), so it loads a job's
// table and flushes its counts once per job rather than once per tile.
__global__ void __launch_bounds__(256) k_srv_half(const SrvJobDev* jobs, const SrvTile* tiles, int ntiles,
                                                  const unsigned long long* tables, int colour, int s) {
    __shared__ __align__(16) unsigned long long s_thr[kMaxTable];
    const int t_lo = (int)((long long)blockIdx.x * ntiles / gridDim.x);
    const int t_hi = (int)((long long)(blockIdx.x + 1) * ntiles / gridDim.x);
    int cur = -1;  // job whose table is loaded and whose counts accumulate
    int nacc = 0, a1 = 0, a2 = 0, a3 = 0;
    for (int ti = t_lo; ti <= t_hi; ++ti) {
        const SrvTile tl = ti < t_hi ? tiles[ti] : SrvTile{-1, 0, 0, 0};
        if (cur >= 0 && tl.job != cur) {  // flush the previous job's counts
            const SrvJobDev& P = jobs[cur];
            long long dP, dM, dQ;
            if (P.model == 0) {
                ising_deltas<4>(nacc, a1, a2, dP, dM);
                dQ = 0;
            } else {
                dP = a1;
                dM = a2;
                dQ = a3;
            }
            long long v[4] = {dP, dM, dQ, (long long)nacc};
            unsigned long long* const dst[4] = {(unsigned long long*)&P.series[3 * s],
                                                (unsigned long long*)&P.series[3 * s + 1],
                                                (unsigned long long*)&P.series[3 * s + 2], P.acc};
            block_add_atomic<4>(v, dst);
            nacc = a1 = a2 = a3 = 0;
            cur = -1;
        }
        if (ti == t_hi) break;
        const SrvJobDev J = jobs[tl.job];
        if (s >= J.todo) continue;  // uniform over the block
        if (cur != tl.job) {
            __syncthreads();
            for (int i = threadIdx.x; i < kMaxTable; i += blockDim.x) {
                const unsigned long long x = tables[(size_t)tl.job * kMaxTable + i];
                s_thr[i] = J.model == 0 ? ising_tab_entry(x, i, 4, J.hb != 0) : x;
            }
            __syncthreads();
            cur = tl.job;
        }
        const unsigned long long t = J.t0 + (unsigned long long)s;
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
    }
}

// ------------------------------------------------------------- resident loop --
// In the resident mode one cooperative kernel keeps running while jobs come and go: every
// round it runs one sweep (both colours) of every armed canonical job on blocks 1..; block 0
// meanwhile takes the jobs the host has armed in a mailbox in pinned host memory and prepares
// the next round, and after the round's last barrier it publishes the jobs that finished.  The host only admits,
// arms and retires jobs; it never waits for the kernel.  Every wait is bounded: the grid
// barriers by spin_limit polls (then the kernel leaves with kLoopTimeout), and a round with no
// job to run by idle_limit polls of about 1 us (then the kernel leaves with kLoopIdle and the
// host launches it again when work arrives).
// Mailbox words live in pinned host memory: system-scope loads and stores.
__device__ __forceinline__ unsigned mb_ld(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long mb_ld64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void mb_st(unsigned* p, unsigned v) {
    asm volatile("st.relaxed.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void mb_st64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

constexpr int kSrvSlots = 256;
static_assert(sizeof(SrvJobDev) % 8 == 0, "SrvJobDev is copied in 8-byte words");
enum LoopStatus : unsigned { kLoopRunning = 0, kLoopStopped = 1, kLoopIdle = 2, kLoopTimeout = 3 };

struct SrvSlotDesc {
    SrvJobDev job;  // series: the job's per-sweep rows (sweep t at 3t); todo: its sweeps
    unsigned long long table[kMaxTable];
};

// Shared by host and device (pinned, mapped).  The host writes a slot's descriptor, then its
// generation, then bumps arm_seq; the device reads arm_seq, then the generations and slots.
struct SrvMailbox {
    unsigned int arm_seq;                 // host: bumped after arming or cancelling slots
    unsigned int stop;                    // host: leave the loop at the end of the round
    unsigned int status;                  // device: LoopStatus of the launch
    unsigned int pad;
    unsigned long long rounds;            // device: rounds run by the current launch
    unsigned int gen[kSrvSlots];          // host: generation of the job armed in the slot (0: none)
    unsigned int cancel[kSrvSlots];       // host: generation to drop before it ends
    unsigned int finished[kSrvSlots];     // device: generation whose run ended (done or dropped)
    unsigned int pad2[kSrvSlots];
    unsigned long long done[kSrvSlots];   // device: sweeps completed by the slot's job
    SrvSlotDesc slots[kSrvSlots];
};

struct SrvRound {
    int n, exit;
    int nbig;                             // entries 0 .. nbig-1 sweep one sweep over the grid
    int nb_solo;                          // blocks that run the small entries nbig .. n-1
    int slot[kSrvSlots];
    int per[kSrvSlots];                   // chunks per tile of the slot's job
    int tile0[kSrvSlots + 1];             // first tile of each big entry; tile0[nbig] = their tiles
    int ks[kSrvSlots];                    // sweeps of each entry in this round (1 for big entries)
    unsigned long long t[kSrvSlots];      // first sweep of each entry in this round
};

struct SrvLoop {
    SrvJobDev jobs[kSrvSlots];
    unsigned long long tables[kSrvSlots][kMaxTable];
    unsigned int gen[kSrvSlots];          // generation taken into each slot
    int fin[kSrvSlots];                   // slots whose job ended in this round
    int nfin;
    unsigned int seen_seq;
    unsigned int reason;                  // exit reason (LoopStatus)
    unsigned int bar[4];                  // grid barrier: arrivals, generation, error
    SrvRound round[2];
};

// Block 0, after its share of the round: the next round's job list (every job one sweep on,
// jobs that ended or were cancelled out), newly armed jobs copied in from the mailbox, and,
// when there is nothing to run, a bounded wait for work.  The host bumps arm_seq after every
// change it makes (arm, cancel, stop), so a round in which nothing changed reads one word of
// host memory; the slots are scanned in parallel only after a change.
constexpr int kSoloChunks = 512;     // jobs with at most this many chunks per colour (one pass of
                                     // a 512-thread block) run on blocks of their own
constexpr int kSoloMaxSweeps = 64;   // at most this many sweeps of a small job per round

__device__ void srv_leader(SrvLoop* L, SrvMailbox* mb, long long r, long long idle_limit) {
    __shared__ int s_n, s_changed, s_stop;
    __shared__ unsigned s_seq;
    __shared__ unsigned s_new[kSrvSlots];
    __shared__ unsigned char s_cancel[kSrvSlots];
    const SrvRound* R = &L->round[r & 1];
    SrvRound* X = &L->round[(r + 1) & 1];
    if (threadIdx.x == 0) s_stop = 0;
    for (long long polls = 0;; ++polls) {
        if (threadIdx.x == 0) {
            s_seq = mb_ld(&mb->arm_seq);
            s_changed = s_seq != L->seen_seq;
            if (s_changed) s_stop = (int)mb_ld(&mb->stop);
            __threadfence_system();
        }
        __syncthreads();
        if (s_changed) {
            for (int sl = threadIdx.x; sl < kSrvSlots; sl += blockDim.x) {
                const unsigned g = mb_ld(&mb->gen[sl]);
                const unsigned c = mb_ld(&mb->cancel[sl]);
                s_cancel[sl] = (c != 0u && c == L->gen[sl]) ? 1 : 0;
                s_new[sl] = (g != 0u && g != L->gen[sl]) ? g : 0u;
            }
        } else if (polls == 0) {
            for (int sl = threadIdx.x; sl < kSrvSlots; sl += blockDim.x) {
                s_cancel[sl] = 0;
                s_new[sl] = 0u;
            }
        }
        __syncthreads();
        if (polls == 0 && threadIdx.x == 0) {  // the jobs that go on
            int n = 0, nf = 0;
            for (int k = 0; k < R->n; ++k) {
                const int sl = R->slot[k];
                const unsigned long long t1 = R->t[k] + (unsigned long long)R->ks[k];
                if (t1 >= (unsigned long long)L->jobs[sl].todo || s_cancel[sl]) {
                    L->fin[nf++] = sl;
                    continue;
                }
                X->slot[n] = sl;
                X->t[n] = t1;
                ++n;
            }
            L->nfin = nf;
            s_n = n;
        }
        __syncthreads();
        if (s_changed) {
            for (int sl = threadIdx.x; sl < kSrvSlots; sl += blockDim.x) {
                const unsigned g = s_new[sl];
                if (!g) continue;
                L->gen[sl] = g;
                __threadfence_system();  // the descriptor was written before the generation
                if (mb_ld(&mb->cancel[sl]) == g) {  // cancelled before it started
                    mb_st(&mb->finished[sl], g);
                    continue;
                }
                const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&mb->slots[sl]);
                unsigned long long* dj = reinterpret_cast<unsigned long long*>(&L->jobs[sl]);
                for (int w = 0; w < (int)(sizeof(SrvJobDev) / 8); ++w) dj[w] = mb_ld64(src + w);
                const unsigned long long* st = src + sizeof(SrvJobDev) / 8;
                for (int w = 0; w < kMaxTable; ++w) L->tables[sl][w] = mb_ld64(st + w);
                const int k = atomicAdd(&s_n, 1);
                X->slot[k] = sl;
                X->t[k] = 0;
            }
            __syncthreads();
            if (threadIdx.x == 0) L->seen_seq = s_seq;
        }
        __syncthreads();
        // wait for work only in an empty round: a round that still runs jobs publishes them first
        if (s_n > 0 || s_stop || R->n > 0 || polls >= idle_limit) break;
        if (threadIdx.x == 0) __nanosleep(1000);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int n = s_n;
        // big entries first (one sweep per round, tiles spread over the grid), then the small
        // ones (a colour within one pass of a block): those run ks sweeps per round each on a
        // block of their own, with block barriers between the colours instead of the grid
        // barrier, so a small job with many sweeps is not held to one sweep per round
        int nbig = 0;
        for (int k = 0; k < n; ++k) {
            const SrvJobDev& J = L->jobs[X->slot[k]];
            if (J.cpr * J.rows > kSoloChunks) {
                const int sl = X->slot[k];
                const unsigned long long tk = X->t[k];
                X->slot[k] = X->slot[nbig];
                X->t[k] = X->t[nbig];
                X->slot[nbig] = sl;
                X->t[nbig] = tk;
                ++nbig;
            }
        }
        const int nb = gridDim.x > 1 ? (int)gridDim.x - 1 : 1;
        if (nbig > 0 && nb < 2) nbig = n;  // no block to spare: every job sweeps over the grid
        int acc = 0;
        for (int k = 0; k < nbig; ++k) {
            const SrvJobDev& J = L->jobs[X->slot[k]];
            const int per = (int)blockDim.x * (16 / J.V);  // one chunk per thread and 16 / V sites
            const int nch = J.cpr * J.rows;
            X->per[k] = per;
            X->tile0[k] = acc;
            X->ks[k] = 1;
            acc += (nch + per - 1) / per;
        }
        X->tile0[nbig] = acc;
        const int nsolo = n - nbig;
        // the small jobs take up to a quarter of the blocks beside big jobs (all of them
        // otherwise).  A small job's sweep is two block passes, a big block's round two colours
        // of its share of the big tiles: the small jobs get as many sweeps per round as fit in
        // that time.  (Sizing their share to one or two sweeps per round instead kept more
        // blocks on the big jobs but let the small ones' passes hold rounds up: 251 against 258
        // attempts/ns and a p50 of 0.36 against 0.31 s on the saturated stream.)
        const int nb_solo = nsolo == 0 ? 0 : (nbig == 0 ? min(nsolo, nb) : min(nsolo, max(1, nb / 4)));
        const int per_block = nb_solo > 0 ? (nsolo + nb_solo - 1) / nb_solo : 1;
        const int big_steps = nbig > 0 ? (acc + (nb - nb_solo) - 1) / (nb - nb_solo) : 0;
        const int K = nbig == 0 ? kSoloMaxSweeps : max(1, min(kSoloMaxSweeps, big_steps / per_block));
        for (int k = nbig; k < n; ++k) {
            const unsigned long long left = (unsigned long long)L->jobs[X->slot[k]].todo - X->t[k];
            X->ks[k] = (int)(left < (unsigned long long)K ? (left > 0 ? left : 1) : K);
            X->per[k] = 0;
        }
        X->nbig = nbig;
        X->nb_solo = nb_solo;
        X->n = n;
        X->exit = (s_stop || (n == 0 && R->n == 0)) ? 1 : 0;
        L->reason = s_stop ? kLoopStopped : (X->exit ? kLoopIdle : kLoopRunning);
    }
    __syncthreads();
}

// All ks sweeps of round entry k (a small job: a colour within one pass of the block) on
// one block: both colours of every sweep, a block barrier between them, the sweep's counts
// flushed to its series slot.
__device__ void srv_solo(SrvLoop* L, const SrvRound* R, int k, unsigned long long* s_thr) {
    const int sl = R->slot[k];
    const SrvJobDev J = L->jobs[sl];
    __syncthreads();
    for (int i = threadIdx.x; i < kMaxTable; i += blockDim.x) {
        const unsigned long long x = L->tables[sl][i];
        s_thr[i] = J.model == 0 ? ising_tab_entry(x, i, 4, J.hb != 0) : x;
    }
    __syncthreads();
    SrvTile tl;
    tl.job = sl;
    tl.c_begin = 0;
    tl.c_end = J.cpr * J.rows;
    tl.pad = 0;
    const int key = J.V * 4 + J.model * 2 + J.hb;
    for (int s = 0; s < R->ks[k]; ++s) {
        const unsigned long long t = R->t[k] + (unsigned long long)s;
        int nacc = 0, a1 = 0, a2 = 0, a3 = 0;
        for (int colour = 0; colour < 2; ++colour) {
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
            __syncthreads();  // this colour's spins are written before the other colour reads them
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
        unsigned long long* const dst[4] = {(unsigned long long*)&J.series[3 * t],
                                            (unsigned long long*)&J.series[3 * t + 1],
                                            (unsigned long long*)&J.series[3 * t + 2], J.acc};
        block_add_atomic<4>(v, dst);
    }
}

constexpr int kLoopThreads = 512;

__global__ void __launch_bounds__(kLoopThreads, 1) k_srv_loop(SrvLoop* L, SrvMailbox* mb, long long spin_limit,
                                                              long long idle_limit) {
    __shared__ __align__(16) unsigned long long s_thr[kMaxTable];
    __shared__ unsigned s_bgen;
    if (threadIdx.x == 0) s_bgen = ld_acquire(&L->bar[1]);
    __syncthreads();
    unsigned gen = s_bgen;
    for (long long r = 0;; ++r) {
        const SrvRound* R = &L->round[r & 1];
        if (R->exit) break;
        const int n = R->nbig;  // the big entries; the small ones are R->nbig .. R->n - 1
        const int total = R->tile0[n];
        const int nb_big = (int)gridDim.x - 1 - R->nb_solo;
        for (int colour = 0; colour < 2; ++colour) {
            // block 0 prepares the next round while the others sweep; it sweeps no tiles
            if (colour == 0 && blockIdx.x == 0) srv_leader(L, mb, r, idle_limit);
            // the small entries: each of the last nb_solo blocks runs all ks sweeps of its
            // share of them during colour 0, a block barrier between the colours
            if (colour == 0 && blockIdx.x > nb_big) {
                const int sb = (int)blockIdx.x - 1 - nb_big;
                const int nsolo = R->n - n;
                const int k_lo = n + (int)((long long)sb * nsolo / R->nb_solo);
                const int k_hi = n + (int)((long long)(sb + 1) * nsolo / R->nb_solo);
                for (int k = k_lo; k < k_hi; ++k) srv_solo(L, R, k, s_thr);
            }
            // every big-job block takes an equal contiguous range of the round's tiles, so
            // consecutive tiles mostly belong to one job: its table is loaded and its counts
            // are flushed (one block reduction, four atomics) once per job, not per tile
            if (blockIdx.x > 0 && blockIdx.x <= nb_big) {
                const int nb = nb_big;
                const int t_lo = (int)((long long)(blockIdx.x - 1) * total / nb);
                const int t_hi = (int)((long long)blockIdx.x * total / nb);
                int lo = 0, hi = n - 1;  // the job of tile t_lo
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (R->tile0[mid] <= t_lo) lo = mid;
                    else hi = mid - 1;
                }
                int cur = -1;  // job index whose table is loaded and whose counts accumulate
                int nacc = 0, a1 = 0, a2 = 0, a3 = 0;
                for (int ti = t_lo; ti <= t_hi; ++ti) {
                    while (ti < t_hi && R->tile0[lo + 1] <= ti) ++lo;
                    if (cur >= 0 && (ti == t_hi || lo != cur)) {  // flush the previous job's counts
                        const SrvJobDev& P = L->jobs[R->slot[cur]];
                        const unsigned long long tp = R->t[cur];
                        long long dP, dM, dQ;
                        if (P.model == 0) {
                            ising_deltas<4>(nacc, a1, a2, dP, dM);
                            dQ = 0;
                        } else {
                            dP = a1;
                            dM = a2;
                            dQ = a3;
                        }
                        long long v[4] = {dP, dM, dQ, (long long)nacc};
                        unsigned long long* const dst[4] = {(unsigned long long*)&P.series[3 * tp],
                                                            (unsigned long long*)&P.series[3 * tp + 1],
                                                            (unsigned long long*)&P.series[3 * tp + 2], P.acc};
                        block_add_atomic<4>(v, dst);
                        nacc = a1 = a2 = a3 = 0;
                        cur = -1;
                    }
                    if (ti == t_hi) break;
                    const int sl = R->slot[lo];
                    const SrvJobDev J = L->jobs[sl];
                    if (cur != lo) {
                        __syncthreads();
                        for (int i = threadIdx.x; i < kMaxTable; i += blockDim.x) {
                            const unsigned long long x = L->tables[sl][i];
                            s_thr[i] = J.model == 0 ? ising_tab_entry(x, i, 4, J.hb != 0) : x;
                        }
                        __syncthreads();
                        cur = lo;
                    }
                    SrvTile tl;
                    tl.job = sl;
                    tl.c_begin = (ti - R->tile0[lo]) * R->per[lo];
                    tl.c_end = min(J.cpr * J.rows, tl.c_begin + R->per[lo]);
                    tl.pad = 0;
                    const unsigned long long t = R->t[lo];
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
                }
            }
            if (!grid_sync(L->bar, gridDim.x, gen, spin_limit)) {
                if (blockIdx.x == 0 && threadIdx.x == 0) {
                    __threadfence_system();
                    mb_st(&mb->status, kLoopTimeout);
                }
                return;
            }
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            // the jobs that ended in this round are complete on the device: publish them
            const SrvRound* X = &L->round[(r + 1) & 1];
            __threadfence_system();
            for (int k = 0; k < L->nfin; ++k) {
                const int sl = L->fin[k];
                mb_st64(&mb->done[sl], (unsigned long long)L->jobs[sl].todo);
                mb_st(&mb->finished[sl], L->gen[sl]);
            }
            if ((r & 15) == 0) {  // progress, every 16 rounds
                for (int k = 0; k < X->n; ++k) mb_st64(&mb->done[X->slot[k]], X->t[k]);
                mb_st64(&mb->rounds, (unsigned long long)r + 1);
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        __threadfence_system();
        mb_st(&mb->status, L->reason);
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
    // resident mode
    size_t pool_off = 0, pool_bytes = 0;  // the job's block of the server arena
    int slot = -1;                        // mailbox slot while armed
    unsigned gen = 0;                     // generation armed in the slot
    cudaEvent_t ready = nullptr;          // initialisation done on the admin stream
    bool armed = false;
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
    // resident mode (mcx_server_start): one persistent kernel sweeps the canonical jobs
    bool resident = false;
    mcx_ctx* admin = nullptr;          // its own stream for initialisation and results
    cudaStream_t lstream = nullptr;    // the loop kernel's stream
    cudaEvent_t ldone = nullptr;
    bool lrunning = false;
    int loop_grid = 0;
    uint64_t loop_launches = 0;
    unsigned last_status = 0;
    long long spin_limit = 1ll << 24, idle_limit = 100000;
    SrvMailbox* mb = nullptr;          // pinned, mapped
    SrvMailbox* mb_dev = nullptr;
    SrvLoop* d_loop = nullptr;
    char* arena = nullptr;
    size_t arena_bytes = 0;
    std::map<size_t, size_t> free_blocks;  // offset -> bytes, coalesced
    std::vector<SrvJob*> slot_job;
    unsigned gen_next = 1;
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

// Bytes of a job's block in the resident arena: colour arrays, staging, (state, counter),
// per-sweep rows, and ln g / H for Multicanonical jobs, each piece 256-byte aligned.
size_t up256(size_t x) { return (x + 255) / 256 * 256; }
size_t carve_bytes(const mcx_job& j) {
    const size_t N = (size_t)j.L[0] * j.L[1];
    size_t b = 2 * up256(N / 2) + up256(N) + 256 + up256((size_t)j.nsweeps * 24);
    if (j.kind == MCX_JOB_MULTICANONICAL) b += 2 * up256((size_t)j.nbins * 8);
    return b;
}

bool pool_alloc(mcx_server* s, size_t bytes, size_t* off) {
    for (auto it = s->free_blocks.begin(); it != s->free_blocks.end(); ++it)
        if (it->second >= bytes) {
            *off = it->first;
            const size_t rest = it->second - bytes;
            const size_t o2 = it->first + bytes;
            s->free_blocks.erase(it);
            if (rest) s->free_blocks[o2] = rest;
            return true;
        }
    return false;
}

void pool_free(mcx_server* s, size_t off, size_t bytes) {
    auto it = s->free_blocks.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != s->free_blocks.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        s->free_blocks.erase(nx);
    }
    if (it != s->free_blocks.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            s->free_blocks.erase(it);
        }
    }
}

// A lattice (and flat-histogram tables) laid out in the job's arena block, on the admin
// context: the library's lattice routines run on it unchanged and never allocate.
void carve_job(mcx_server* s, SrvJob* j) {
    const mcx_job& sp = j->spec;
    char* b = s->arena + j->pool_off;
    const size_t N = (size_t)sp.L[0] * sp.L[1];
    mcx_lattice* L = new mcx_lattice();
    L->ctx = s->admin;
    L->model = (mcx_model)sp.model;
    L->layout = MCX_LAYOUT_INT8;
    L->dim = 2;
    L->L[0] = sp.L[0];
    L->L[1] = sp.L[1];
    L->L[2] = 1;
    L->J = sp.J;
    L->D = sp.D;
    L->h = sp.h;
    L->N = (int64_t)N;
    L->W = sp.L[0] / 2;
    L->rows = sp.L[1];
    L->d_col[0] = (int8_t*)b;
    b += up256(N / 2);
    L->d_col[1] = (int8_t*)b;
    b += up256(N / 2);
    L->d_lin = (int8_t*)b;
    b += up256(N);
    L->d_state = (int64_t*)b;
    L->d_acc = (unsigned long long*)(b + 32);
    b += 256;
    L->d_series = (int64_t*)b;
    L->series_cap = sp.nsweeps;
    b += up256((size_t)sp.nsweeps * 24);
    j->lat = L;
    if (sp.kind == MCX_JOB_MULTICANONICAL) {
        mcx_flathist* F = new mcx_flathist();
        F->ctx = s->admin;
        F->start = sp.bin_start;
        F->step = sp.bin_step;
        F->nbins = sp.nbins;
        F->d_lnw = (double*)b;
        b += up256((size_t)sp.nbins * 8);
        F->d_H = (unsigned long long*)b;
        j->fh = F;
    }
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
    if (s->resident) {
        delete j->lat;  // carved from the arena: no device memory of its own
        delete j->fh;
        if (j->pool_bytes) pool_free(s, j->pool_off, j->pool_bytes);
        j->pool_bytes = 0;
        if (j->ready) cudaEventDestroy(j->ready);
        j->ready = nullptr;
    } else {
        if (j->lat) mcx_lattice_destroy(j->lat);
        if (j->fh) mcx_flathist_destroy(j->fh);
    }
    j->lat = nullptr;
    j->fh = nullptr;
    s->used -= j->bytes;
}

mcx_status admit(mcx_server* s, SrvJob* j) {
    const mcx_job& sp = j->spec;
    if (s->resident) {
        carve_job(s, j);
    } else {
        const int32_t L[3] = {sp.L[0], sp.L[1], 1};
        MCX_CHECK(mcx_lattice_create(s->ctx, (mcx_model)sp.model, 2, L, MCX_LAYOUT_INT8, sp.J, sp.D, sp.h, &j->lat));
    }
    s->used += j->bytes;
    s->peak = std::max(s->peak, s->used);
    cudaStream_t st0 = j->lat->ctx->stream;
    MCX_CHECK(mcx_init_random(j->lat, sp.seed, sp.stream));
    MCX_CHECK(ensure_series(j->lat, sp.nsweeps));
    MCX_CUDA(cudaMemsetAsync(j->lat->d_series, 0, (size_t)sp.nsweeps * 24, st0));
    MCX_CUDA(cudaMemsetAsync(j->lat->d_acc, 0, 8, st0));
    if (sp.kind == MCX_JOB_CANONICAL) {
        MCX_CHECK(build_table(j->lat, (mcx_algorithm)sp.alg, sp.beta, &j->table));
        if (s->resident) {
            MCX_CUDA(cudaEventCreateWithFlags(&j->ready, cudaEventDisableTiming));
            MCX_CUDA(cudaEventRecord(j->ready, st0));
        }
    } else {
        if (s->resident) {
            MCX_CUDA(cudaMemsetAsync(j->fh->d_lnw, 0, (size_t)sp.nbins * 8, st0));
            MCX_CUDA(cudaMemsetAsync(j->fh->d_H, 0, (size_t)sp.nbins * 8, st0));
        } else {
            MCX_CHECK(mcx_flathist_create(s->ctx, sp.bin_start, sp.bin_step, sp.nbins, &j->fh));
        }
        if (!j->lnw0.empty())
            MCX_CUDA(cudaMemcpyAsync(j->fh->d_lnw, j->lnw0.data(), j->lnw0.size() * 8, cudaMemcpyHostToDevice, st0));
        long long st[3];
        MCX_CUDA(cudaMemcpyAsync(st, j->lat->d_state, 24, cudaMemcpyDeviceToHost, st0));
        MCX_CUDA(cudaStreamSynchronize(st0));
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
    mcx_ctx* ctx = j->lat->ctx;  // the server's context, or in the resident mode its admin context
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
    // the walkers' lattices were initialised on the context (or admin) stream
    MCX_CUDA(cudaStreamSynchronize(s->resident ? s->admin->stream : s->ctx->stream));
    MCX_CHECK(grow(s, &s->d_walkers, &s->cap_walkers, s->mwalk.size()));
    MCX_CUDA(cudaMemcpyAsync(s->d_walkers, s->mwalk.data(), s->mwalk.size() * sizeof(FHWalker), cudaMemcpyHostToDevice,
                             s->mstream));
    MCX_CHECK(launch_flathist_on(s->ctx, s->mstream, s->d_walkers, (int)s->mwalk.size()));
    MCX_CUDA(cudaEventRecord(s->mdone, s->mstream));
    s->minflight = true;
    return MCX_OK;
}

// ---------------------------------------------------------------- resident pump --
unsigned vload(const unsigned* p) { return __atomic_load_n(p, __ATOMIC_ACQUIRE); }
void vstore(unsigned* p, unsigned v) { __atomic_store_n(p, v, __ATOMIC_RELEASE); }

// Writes the job's descriptor into a free mailbox slot, then its generation, then bumps the
// arm sequence the loop kernel watches.
mcx_status arm(mcx_server* s, SrvJob* j) {
    int sl = -1;
    for (int k = 0; k < kSrvSlots; ++k)
        if (!s->slot_job[k]) {
            sl = k;
            break;
        }
    if (sl < 0) return MCX_OK;  // every slot busy: armed at a later step
    const mcx_lattice* L = j->lat;
    SrvSlotDesc& d = s->mb->slots[sl];
    std::memset(&d, 0, sizeof(d));
    d.job.col[0] = L->d_col[0];
    d.job.col[1] = L->d_col[1];
    d.job.series = (long long*)L->d_series;
    d.job.acc = L->d_acc;
    d.job.W = (int)L->W;
    d.job.Ly = (int)L->L[1];
    d.job.rows = (int)L->rows;
    d.job.V = L->W % 16 == 0 ? 16 : (L->W % 8 == 0 ? 8 : 4);
    d.job.cpr = d.job.W / d.job.V;
    d.job.model = L->model == MCX_ISING ? 0 : 1;
    d.job.hb = j->spec.alg == MCX_HEATBATH;
    d.job.todo = (int)j->spec.nsweeps;
    d.job.k0 = (uint32_t)j->spec.seed;
    d.job.k1 = (uint32_t)(j->spec.seed >> 32);
    d.job.stream = j->spec.stream;
    d.job.m_cpr = d.job.cpr <= 1 ? 0u : (uint32_t)(((1ull << 32) + d.job.cpr - 1) / d.job.cpr);
    d.job.t0 = 0;
    for (int i = 0; i < kMaxTable; ++i) d.table[i] = i < j->table.n ? j->table.thr[i] : 0ull;
    j->gen = s->gen_next++;
    if (s->gen_next == 0) s->gen_next = 1;
    j->slot = sl;
    j->armed = true;
    s->slot_job[sl] = j;
    vstore(&s->mb->cancel[sl], 0u);
    vstore(&s->mb->finished[sl], 0u);
    s->mb->done[sl] = 0;
    std::atomic_thread_fence(std::memory_order_seq_cst);
    vstore(&s->mb->gen[sl], j->gen);
    std::atomic_thread_fence(std::memory_order_seq_cst);
    vstore(&s->mb->arm_seq, s->mb->arm_seq + 1);
    return MCX_OK;
}

mcx_status launch_loop(mcx_server* s) {
    MCX_CUDA(cudaMemsetAsync(s->d_loop, 0, sizeof(SrvLoop), s->lstream));
    vstore(&s->mb->stop, 0u);
    vstore(&s->mb->status, kLoopRunning);
    // a new launch starts with seen_seq = 0: make sure it scans the slots once
    if (s->mb->arm_seq == 0u) vstore(&s->mb->arm_seq, 1u);
    SrvLoop* L = s->d_loop;
    SrvMailbox* mb = s->mb_dev;
    long long spin = s->spin_limit, idle = s->idle_limit;
    void* args[] = {&L, &mb, &spin, &idle};
    MCX_CUDA(cudaLaunchCooperativeKernel((const void*)k_srv_loop, dim3(s->loop_grid), dim3(kLoopThreads), args, 0,
                                         s->lstream));
    MCX_CUDA(cudaEventRecord(s->ldone, s->lstream));
    count_launch(s->ctx);
    s->loop_launches += 1;
    s->lrunning = true;
    return MCX_OK;
}

mcx_status step_resident(mcx_server* s) {
    // 1. the loop kernel: has it left (idle, stopped, or a barrier that gave up)?
    if (s->lrunning) {
        const cudaError_t q = cudaEventQuery(s->ldone);
        if (q == cudaSuccess) {
            s->lrunning = false;
            s->last_status = vload(&s->mb->status);
            if (s->last_status == kLoopTimeout) {
                for (SrvJob* j : s->active)
                    if (j->armed) j->status = MCX_ERR_TIMEOUT;
                return fail(MCX_ERR_TIMEOUT, "serving loop: a grid barrier wait exceeded its limit");
            }
        } else if (q != cudaErrorNotReady) {
            return cuda_fail(q, "serving loop");
        }
    }
    // 2. jobs the loop has finished (or dropped after a cancel)
    std::vector<SrvJob*> still;
    for (SrvJob* j : s->active) {
        if (j->armed && vload(&s->mb->finished[j->slot]) == j->gen) {
            s->slot_job[j->slot] = nullptr;
            j->armed = false;
            vstore(&s->mb->gen[j->slot], 0u);
            if (j->cancel_req) {
                j->state = JOB_CANCELLED;
                j->t_finish = now_s(s->t0);
                release(s, j);
            } else {
                j->done = j->spec.nsweeps;
                MCX_CHECK(finish(s, j));
            }
            continue;
        }
        still.push_back(j);
    }
    s->active.swap(still);
    // 3. admission in arrival order, by slots, HBM budget and room in the arena
    while (!s->pending.empty() && (int)s->active.size() < s->max_jobs) {
        SrvJob* j = s->pending.front();
        if (s->budget && s->used + j->bytes > s->budget) break;
        if (!pool_alloc(s, carve_bytes(j->spec), &j->pool_off)) break;
        j->pool_bytes = carve_bytes(j->spec);
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
    // 4. initialised canonical jobs are armed for the loop
    bool waiting = false;
    for (SrvJob* j : s->active) {
        if (j->spec.kind != MCX_JOB_CANONICAL || j->armed) continue;
        const cudaError_t q = cudaEventQuery(j->ready);
        if (q == cudaSuccess) MCX_CHECK(arm(s, j));
        else if (q != cudaErrorNotReady) return cuda_fail(q, "job initialisation");
    }
    for (SrvJob* j : s->active)
        if (j->armed) waiting = true;
    // 5. Multicanonical jobs on the walker stream
    MCX_CHECK(collect_muca(s));
    if (!s->minflight) {
        for (SrvJob* j : s->deferred) release(s, j);
        s->deferred.clear();
    }
    MCX_CHECK(launch_muca(s));
    // 6. the loop runs while armed jobs wait for it
    if (waiting && !s->lrunning) MCX_CHECK(launch_loop(s));
    s->iterations += 1;
    if (!s->active.empty()) std::this_thread::sleep_for(std::chrono::microseconds(20));  // a pump, not a spin
    return MCX_OK;
}

// Bounded host wait for the loop kernel to leave.
mcx_status wait_loop(mcx_server* s, double seconds) {
    const auto t0 = std::chrono::steady_clock::now();
    while (s->lrunning) {
        const cudaError_t q = cudaEventQuery(s->ldone);
        if (q == cudaSuccess) {
            s->lrunning = false;
            s->last_status = vload(&s->mb->status);
            break;
        }
        if (q != cudaErrorNotReady) return cuda_fail(q, "serving loop");
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > seconds)
            return fail(MCX_ERR_TIMEOUT, "the serving loop did not stop within %.1f s", seconds);
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
    return MCX_OK;
}

// one scheduling iteration
mcx_status step(mcx_server* s) {
    if (s->resident) return step_resident(s);
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
    if (s->resident && s->lrunning) {
        vstore(&s->mb->stop, 1u);
        std::atomic_thread_fence(std::memory_order_seq_cst);
        vstore(&s->mb->arm_seq, s->mb->arm_seq + 1);
        wait_loop(s, 30.0);
    }
    if (s->lstream) cudaStreamSynchronize(s->lstream);
    if (s->admin) cudaStreamSynchronize(s->admin->stream);
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
    if (s->resident) {
        if (s->d_loop) dev_free(s->ctx, s->d_loop, sizeof(SrvLoop));
        if (s->arena) dev_free(s->ctx, s->arena, s->arena_bytes);
        if (s->mb) cudaFreeHost(s->mb);
        if (s->ldone) cudaEventDestroy(s->ldone);
        if (s->lstream) cudaStreamDestroy(s->lstream);
        if (s->admin) mcx_ctx_destroy(s->admin);
    }
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
    res->sweeps_done = j->armed ? (int64_t)s->mb->done[j->slot] : j->done;
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
        if (j->armed) {  // the loop drops it at the end of a round; retired at a later step
            j->cancel_req = true;
            vstore(&s->mb->cancel[j->slot], j->gen);
            std::atomic_thread_fence(std::memory_order_seq_cst);
            vstore(&s->mb->arm_seq, s->mb->arm_seq + 1);
            return MCX_OK;
        }
        if (s->resident) {  // admitted, not armed yet: its initialisation may still run
            MCX_CUDA(cudaStreamSynchronize(s->admin->stream));
            s->active.erase(std::find(s->active.begin(), s->active.end(), j));
            if (s->minflight) s->deferred.push_back(j);
            else release(s, j);
            j->state = JOB_CANCELLED;
            j->t_finish = now_s(s->t0);
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

MCX_API mcx_status mcx_server_start(mcx_server* s) {
    if (!s) return fail(MCX_ERR_INVALID_ARG, "server is NULL");
    if (s->resident) return MCX_OK;
    if (!s->budget) return fail(MCX_ERR_INVALID_ARG, "the resident loop needs an HBM budget (its job arena)");
    if (s->max_jobs > kSrvSlots) return fail(MCX_ERR_INVALID_ARG, "the resident loop has %d job slots", kSrvSlots);
    if (!s->active.empty()) return fail(MCX_ERR_INVALID_ARG, "start the resident loop before admitting jobs");
    mcx_ctx* ctx = s->ctx;
    int coop = 0;
    MCX_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device));
    if (!coop) return fail(MCX_ERR_CUDA, "the device has no cooperative launch");
    int bps = 0;
    MCX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_srv_loop, kLoopThreads, 0));
    if (bps < 1) return fail(MCX_ERR_CUDA, "the serving loop kernel does not fit on an SM");
    // One 512-thread block per SM at most on all but `reserve` SMs: each block holds an SM's
    // whole register file, so at least `reserve` SMs stay empty for the kernels the pump
    // launches beside the loop (initialisation, series prefix, spin gather, walkers) and for
    // any kernel that needs a whole SM; with the loop on every SM those would wait for it.
    const int reserve = std::min(8, ctx->num_sms / 4);
    s->loop_grid = ctx->num_sms - reserve;
    void* p = nullptr;
    MCX_CHECK(dev_alloc(ctx, &p, (size_t)s->budget));
    s->arena = (char*)p;
    s->arena_bytes = (size_t)s->budget;
    s->free_blocks.clear();
    s->free_blocks[0] = s->arena_bytes;
    MCX_CHECK(dev_alloc(ctx, &p, sizeof(SrvLoop)));
    s->d_loop = (SrvLoop*)p;
    MCX_CUDA(cudaHostAlloc((void**)&s->mb, sizeof(SrvMailbox), cudaHostAllocMapped));
    std::memset(s->mb, 0, sizeof(SrvMailbox));
    MCX_CUDA(cudaHostGetDevicePointer((void**)&s->mb_dev, s->mb, 0));
    mcx_config cfg{ctx->device, nullptr, 0};
    MCX_CHECK(mcx_ctx_create(&cfg, &s->admin));
    MCX_CUDA(cudaStreamCreateWithFlags(&s->lstream, cudaStreamNonBlocking));
    MCX_CUDA(cudaEventCreateWithFlags(&s->ldone, cudaEventDisableTiming));
    if (!s->mstream) {
        MCX_CUDA(cudaStreamCreateWithFlags(&s->mstream, cudaStreamNonBlocking));
        MCX_CUDA(cudaEventCreateWithFlags(&s->mdone, cudaEventDisableTiming));
    }
    s->slot_job.assign(kSrvSlots, nullptr);
    // walker descriptors for every slot now: no device allocation may happen while the loop runs
    MCX_CHECK(grow(s, &s->d_walkers, &s->cap_walkers, (size_t)kSrvSlots));
    s->resident = true;
    // Load every kernel the pump launches while the loop runs (initialisation, series prefix,
    // both spin gathers, walker) with small jobs run to completion first: a kernel loaded on
    // first use while the loop kernel holds the device would wait for it.
    mcx_job w{};
    w.model = MCX_ISING;
    w.dim = 2;
    w.L[0] = w.L[1] = 16;
    w.L[2] = 1;
    w.kind = MCX_JOB_CANONICAL;
    w.alg = MCX_METROPOLIS;
    w.beta = 0.4;
    w.J = 1.0;
    w.nsweeps = 2;
    std::vector<int8_t> spins(256);
    std::vector<int64_t> ser(6);
    w.obs_series = ser.data();
    w.final_spins = spins.data();
    uint64_t ids[3] = {0, 0, 0};
    mcx_job wm = w;  // the Multicanonical jobs run first, with no loop kernel on the device
    wm.kind = MCX_JOB_MULTICANONICAL;
    wm.bin_start = -512;
    wm.bin_step = 4;
    wm.nbins = 257;
    std::vector<int64_t> hist(257);
    wm.histogram = hist.data();
    mcx_job wm2 = wm;  // rows of 24 sites: the gather without 16-site vectors
    wm2.L[0] = 24;
    wm2.L[1] = 8;
    wm2.bin_start = -384;
    wm2.nbins = 193;
    const mcx_job* warm[3] = {&wm, &wm2, &w};
    const long long idle = s->idle_limit;
    s->idle_limit = 16;  // the loop leaves as soon as the warm-up job is done
    mcx_status st = MCX_OK;
    const auto t0 = std::chrono::steady_clock::now();
    for (int phase = 0; phase < 3 && st == MCX_OK; ++phase) {
        st = mcx_server_submit(s, warm[phase], &ids[phase]);
        while (st == MCX_OK) {
            st = step_resident(s);
            if (st == MCX_OK && s->active.empty() && s->pending.empty()) {
                st = wait_loop(s, 10.0);
                break;
            }
            if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > 60.0)
                st = fail(MCX_ERR_TIMEOUT, "the serving loop's first jobs did not finish");
        }
    }
    s->idle_limit = idle;
    MCX_CHECK(st);
    for (uint64_t id : ids) {
        auto it = s->jobs.find(id);
        delete it->second;
        s->jobs.erase(it);
    }
    s->jobs_done -= 3;
    s->attempts_done = 0;
    s->peak = s->used;
    return MCX_OK;
}

MCX_API mcx_status mcx_server_stop(mcx_server* s, double timeout_s) {
    if (!s) return fail(MCX_ERR_INVALID_ARG, "server is NULL");
    if (!s->resident || !s->lrunning) return MCX_OK;
    vstore(&s->mb->stop, 1u);
    std::atomic_thread_fence(std::memory_order_seq_cst);
    vstore(&s->mb->arm_seq, s->mb->arm_seq + 1);
    return wait_loop(s, timeout_s);
}

MCX_API mcx_status mcx_server_set_loop_limits(mcx_server* s, int64_t spin_polls, int64_t idle_polls) {
    if (!s || spin_polls < 1 || idle_polls < 0) return fail(MCX_ERR_INVALID_ARG, "bad argument");
    if (idle_polls * 100 >= spin_polls)
        return fail(MCX_ERR_INVALID_ARG, "the idle wait (polls of ~1 us) must stay well below the barrier limit "
                                         "(polls of ~0.1 us): idle_polls * 100 < spin_polls");
    s->spin_limit = spin_polls;
    s->idle_limit = idle_polls;
    return MCX_OK;
}

MCX_API mcx_status mcx_server_loop_info(mcx_server* s, int32_t* resident, int32_t* running, uint32_t* status,
                                        uint64_t* launches, uint64_t* rounds) {
    if (!s) return fail(MCX_ERR_INVALID_ARG, "server is NULL");
    if (resident) *resident = s->resident ? 1 : 0;
    if (running) *running = s->lrunning ? 1 : 0;
    if (status) *status = s->resident ? (s->lrunning ? (unsigned)kLoopRunning : s->last_status) : 0u;
    if (launches) *launches = s->loop_launches;
    if (rounds) *rounds = s->resident ? s->mb->rounds : 0;
    return MCX_OK;
}

MCX_API mcx_status mcx_poll_flag(const uint32_t* flag, uint32_t target, int64_t polls, int64_t sleep_ns) {
    if (!flag || polls < 0 || sleep_ns < 0) return fail(MCX_ERR_INVALID_ARG, "bad argument");
    for (int64_t n = 0;; ++n) {
        if (__atomic_load_n(flag, __ATOMIC_ACQUIRE) >= target) return MCX_OK;
        if (n >= polls) return fail(MCX_ERR_TIMEOUT, "flag stayed below %u for %lld polls", target, (long long)polls);
        if (sleep_ns) std::this_thread::sleep_for(std::chrono::nanoseconds(sleep_ns));
    }
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

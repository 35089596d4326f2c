// mcx_pt.cu -- batched parallel tempering: many Ising replicas of uneven size, their
// checkerboard sweeps and the replica-exchange step.
//
// Two forms with bit-identical results:
//   PERSISTENT: one cooperative launch runs all sweeps of all replicas.  Every warp of
//     the grid owns one chunk range of one replica (built on the host: warps are handed
//     to replicas by cost, and a replica's chunks are split evenly among its warps), so
//     a phase needs no block barrier and no atomic claiming.  Between the colours of
//     a sweep a replica's warps wait only for one another (arrival counter); a
//     bounded grid barrier separates the sweep from the exchange; every
//     block then evaluates the (tiny) exchange step itself, so the new ladder
//     positions need no further barrier.  Per-replica energy deltas are triple
//     buffered so that one sweep's accumulation never meets another's reads.
//   PLAIN: one launch per replica and colour plus one exchange launch per sweep.
//
// Exchange rule: src/algorithms/replica_exchange.jl:110-178 (threads update!): pairs
// (p, p+1) with p = first, first+2, ... where first = stage even ? 0 : 1 (0-based);
// lr = (lw_i(x_j) - lw_i(x_i)) + (lw_j(x_i) - lw_j(x_j)) with lw(x) = -beta*x;
// accept iff lr > 0 || U < exp(lr), evaluated as log(U) < lr with the project log;
// on acceptance the two replicas swap ladder positions (their betas); the stage
// toggles after every exchange step.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <queue>
#include <vector>

#include "mcx_body.cuh"
#include "mcx_cb.cuh"
#include "mcx_device.cuh"
#include "mcx_internal.h"
#include "mcx_sweep.cuh"

namespace mcx {

struct PTReplica {
    long long off[2];  // colour arrays inside the arena
    int W, Ly, Lz, cpr, V, rows;
    int ladder, gpos0, n;  // ladder id, first global position of the ladder, ladder size
    uint32_t m_cpr, m_Ly;  // round-up reciprocals for exact division of small integers
};

struct PTTile {
    int rep, c_begin, c_end, sites;
    int nw;  // persistent spans: warps sharing this replica
    // 3-D plane walk (ze > zb): lane l takes chunk c_begin + l of every plane (while it is
    // below c_end, the plane's chunk count) for the planes zb .. ze-1
    int zb, ze;
};

struct PTArgs {
    int8_t* arena;
    const PTReplica* reps;
    const PTTile* tiles;     // per-block tiles of one replica-colour (plain form)
    const PTTile* spans;     // one chunk range of one replica per warp of the grid (persistent form)
    int nrep, npos, ntiles;
    const unsigned long long* tables;  // [npos][16] for the algorithm of this run (ising_tab_entry form)
    const uint32_t* tables32;          // the same minus 1 (32-bit form, when no entry is 0)
    const double* betas;               // [npos]
    const int* pos_ladder;             // [npos]
    const int* pos_local;              // [npos]
    const int* ladder_n;               // [nladders]
    int32_t* pos;                      // [nrep] ladder position of each replica
    int32_t* stage;
    long long* state;                  // [nrep][2] pair sum, spin sum
    long long* delta;                  // [3][nrep][2]
    unsigned long long* acc;           // [nrep]
    unsigned long long* ex_steps;      // [npos] edge (p, p+1) counted at the global position of p
    unsigned long long* ex_acc;        // [npos]
    long long* series;                 // [nsweeps][nrep][2] or null
    unsigned int* bar;                 // count, generation, error
    unsigned long long* repbar;        // [nrep] colour-0 arrivals of each replica's warps (persistent form)
    double* logu;                      // [2][npos] exchange log-uniforms (persistent form)
    double J, h;
    uint32_t k0, k1;
    unsigned long long sweep0;
    long long nsweeps;
    int every;
    long long spin_limit;
    int series_by_pos;                 // series columns: 0 replicas, 1 global ladder positions
};

// n / d for small n, d: m = ceil(2^32 / d) (exact while n < 2^32 / d); m = 0 encodes d = 1
__device__ __forceinline__ uint32_t fdiv(uint32_t n, uint32_t m) { return m ? __umulhi(n, m) : n; }

// One tile of one replica: chunks [c_begin, c_end) of colour `colour`; `tab` is the
// replica's table in shared memory (64-bit, or 32-bit when T32).
template <int DIM, int V, bool HB, bool T32>
__device__ __forceinline__ void pt_tile(const PTArgs& a, const PTReplica& R, int rep, int c_begin, int c_end,
                                        int colour, unsigned long long sweep, const void* tab, int& nacc, int& nup,
                                        int& isum) {
    constexpr int Z = 2 * DIM;
    constexpr int NW = V / 4;
    int8_t* cur = a.arena + R.off[colour];
    const int8_t* oth = a.arena + R.off[1 - colour];
    const uint32_t w2 = ctr_word2(sweep, colour, P_ACCEPT);
    for (int g = c_begin + (int)threadIdx.x; g < c_end; g += blockDim.x) {
        const int r = (int)fdiv((uint32_t)g, R.m_cpr);
        const int q = g - r * R.cpr;
        const int z = (int)fdiv((uint32_t)r, R.m_Ly);
        const int y = r - z * R.Ly;
        const RowInfo ri = row_info_yz(y, z, R.Ly, R.Lz, colour, DIM);
        Chunk<DIM, V> ch;
        ch.load(cur, oth, R.W, r, q * V, ri);
        const uint32_t c0 = (uint32_t)(((unsigned long long)r * R.W + q * V) >> 2);
        uint32_t af = 0, au = 0, ai = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            uint32_t nbw[Z];
#pragma unroll
            for (int d = 0; d < Z; ++d) nbw[d] = ch.nb[d][w];
            const uint4 rnd = philox10(make_uint4(c0 + w, (uint32_t)sweep, w2, (uint32_t)rep), a.k0, a.k1);
            uint32_t fb;
            if (T32) fb = ising_word32<Z, HB>(nbw, ch.own[w], rnd, (const uint32_t*)tab, af, au, ai);
            else fb = ising_word<Z, HB>(nbw, ch.own[w], rnd, (const unsigned long long*)tab, nacc, nup, isum);
            ch.own[w] ^= fb * 0xFEu;
        }
        if (T32) {
            nacc += hsum8(af);
            nup += hsum8(au);
            isum += hsum16(ai);
        }
        store_row<V>(cur + (long long)r * R.W + q * V, ch.own);
    }
}

// Warp-level sum of N int64 values and one atomic per value per warp (no block
// barrier, so a block can move from tile to tile without synchronising).
template <int N>
__device__ __forceinline__ void warp_add_atomic(long long (&v)[N], unsigned long long* const (&dst)[N]) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
        long long x = v[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
        if ((threadIdx.x & 31) == 0 && x != 0) atomicAdd(dst[j], (unsigned long long)x);
    }
}

// One warp's chunk range [c_begin, c_end) of one replica: lanes take consecutive chunks
// (coalesced rows), no block barrier; deltas reduced over the warp.
template <int DIM, int V, bool HB, bool T32>
__device__ __forceinline__ void pt_span(const PTArgs& a, const PTReplica& R, int rep, int c_begin, int c_end,
                                        int colour, unsigned long long sweep, const void* tab, int lane, int& nacc,
                                        int& nup, int& isum) {
    constexpr int Z = 2 * DIM;
    constexpr int NW = V / 4;
    int8_t* cur = a.arena + R.off[colour];
    const int8_t* oth = a.arena + R.off[1 - colour];
    const uint32_t w2 = ctr_word2(sweep, colour, P_ACCEPT);
    for (int g = c_begin + lane; g < c_end; g += 32) {
        const int r = (int)fdiv((uint32_t)g, R.m_cpr);
        const int q = g - r * R.cpr;
        const int z = (int)fdiv((uint32_t)r, R.m_Ly);
        const int y = r - z * R.Ly;
        const RowInfo ri = row_info_yz(y, z, R.Ly, R.Lz, colour, DIM);
        Chunk<DIM, V> ch;
        ch.load(cur, oth, R.W, r, q * V, ri);
        const uint32_t c0 = (uint32_t)(((unsigned long long)r * R.W + q * V) >> 2);
        uint32_t af = 0, au = 0, ai = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            uint32_t nbw[Z];
#pragma unroll
            for (int d = 0; d < Z; ++d) nbw[d] = ch.nb[d][w];
            const uint4 rnd = philox10(make_uint4(c0 + w, (uint32_t)sweep, w2, (uint32_t)rep), a.k0, a.k1);
            uint32_t fb;
            if (T32) fb = ising_word32<Z, HB>(nbw, ch.own[w], rnd, (const uint32_t*)tab, af, au, ai);
            else fb = ising_word<Z, HB>(nbw, ch.own[w], rnd, (const unsigned long long*)tab, nacc, nup, isum);
            ch.own[w] ^= fb * 0xFEu;
        }
        if (T32) {
            nacc += hsum8(af);
            nup += hsum8(au);
            isum += hsum16(ai);
        }
        store_row<V>(cur + (long long)r * R.W + q * V, ch.own);
    }
}

// 3-D plane walk of one warp: lane l takes chunk pc = c_plane + l of a plane (row y = pc /
// cpr, chunk q) in every plane zb .. ze-1, in order; the other colour's planes z and z+1 of
// that row are carried to the next plane as its z-1 and z neighbours, so a plane costs the
// own words, the other colour's rows y+1 and y-1 and plane z+1, and one edge byte.  The 32
// lanes read 32 consecutive chunks of a plane (one coalesced range).  Same stream, same
// results as pt_span.
template <int V, bool HB, bool T32>
__device__ __forceinline__ void pt_zwalk(const PTArgs& a, const PTReplica& R, int rep, int c_plane, int c_lim, int zb,
                                         int ze, int colour, unsigned long long sweep, const void* tab, int lane,
                                         int& nacc, int& nup, int& isum) {
    constexpr int NW = V / 4;
    const int pc = c_plane + lane;
    if (pc >= c_lim) return;
    const int y = (int)fdiv((uint32_t)pc, R.m_cpr);
    const int q = pc - y * R.cpr;
    const int k0 = q * V;
    const long long W = R.W;
    const long long PS = (long long)R.Ly * W;  // bytes of one plane of a colour array
    const long long dyp = (y + 1 == R.Ly ? -(long long)y : 1ll) * W;
    const long long dym = (y == 0 ? (long long)(R.Ly - 1) : -1ll) * W;
    const int keL = k0 == 0 ? R.W - 1 : k0 - 1;
    const int keR = k0 + V == R.W ? 0 : k0 + V;
    int8_t* cp = a.arena + R.off[colour] + (long long)zb * PS + (long long)y * W + k0;
    const int8_t* op = a.arena + R.off[1 - colour] + (long long)zb * PS + (long long)y * W;  // row y of plane z
    uint32_t c0 = (uint32_t)((((unsigned long long)zb * R.Ly + y) * (unsigned long long)R.W + k0) >> 2);
    int p = (y + zb + colour) & 1;
    const SweepKey key{sweep, a.k0, a.k1, (uint32_t)rep};
    const uint32_t w2 = ctr_word2(sweep, colour, P_ACCEPT);
    uint32_t zm[NW], mid[NW], zp[NW];
    load_row<V>(op + (zb == 0 ? (long long)(R.Lz - 1) * PS : -PS) + k0, zm);
    load_row<V>(op + k0, mid);
    for (int z = zb; z < ze; ++z) {
        load_row<V>(op + (z + 1 == R.Lz ? -(long long)z * PS : PS) + k0, zp);
        Chunk<3, V> ch;
        load_row<V>(cp, ch.own);
        load_row<V>(op + dyp + k0, ch.nb[1]);
        load_row<V>(op + dym + k0, ch.nb[2]);
        const uint32_t edge = (uint32_t)(uint8_t)op[p == 0 ? keL : keR];
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            ch.nb[0][w] = mid[w];
            ch.nb[4][w] = zp[w];
            ch.nb[5][w] = zm[w];
        }
        if (p == 0) {
#pragma unroll
            for (int w = 0; w < NW; ++w)
                ch.nb[3][w] = __funnelshift_l(w == 0 ? (edge << 24) : mid[w - 1], mid[w], 8);
        } else {
#pragma unroll
            for (int w = 0; w < NW; ++w) ch.nb[3][w] = __funnelshift_r(mid[w], w == NW - 1 ? edge : mid[w + 1], 8);
        }
        ising_chunk<3, V, HB, T32>(ch, c0, key, w2, (const unsigned long long*)tab, (const uint32_t*)tab, nacc, nup,
                                   isum);
        store_row<V>(cp, ch.own);
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            zm[w] = mid[w];
            mid[w] = zp[w];
        }
        cp += PS;
        op += PS;
        c0 += (uint32_t)(PS >> 2);
        p ^= 1;
    }
}

template <int DIM, bool HB, bool T32>
__device__ __forceinline__ void pt_run_span(const PTArgs& a, const PTTile& sp, int colour, unsigned long long sweep,
                                            long long* dcur, const void* thr, int lane) {
    const PTReplica R = a.reps[sp.rep];
    int nacc = 0, nup = 0, isum = 0;
    if (DIM == 3 && sp.ze > sp.zb) {
        if (R.V == 16) pt_zwalk<16, HB, T32>(a, R, sp.rep, sp.c_begin, sp.c_end, sp.zb, sp.ze, colour, sweep, thr, lane, nacc, nup, isum);
        else if (R.V == 8) pt_zwalk<8, HB, T32>(a, R, sp.rep, sp.c_begin, sp.c_end, sp.zb, sp.ze, colour, sweep, thr, lane, nacc, nup, isum);
        else pt_zwalk<4, HB, T32>(a, R, sp.rep, sp.c_begin, sp.c_end, sp.zb, sp.ze, colour, sweep, thr, lane, nacc, nup, isum);
    } else if (R.V == 16) {
        pt_span<DIM, 16, HB, T32>(a, R, sp.rep, sp.c_begin, sp.c_end, colour, sweep, thr, lane, nacc, nup, isum);
    } else if (R.V == 8) {
        pt_span<DIM, 8, HB, T32>(a, R, sp.rep, sp.c_begin, sp.c_end, colour, sweep, thr, lane, nacc, nup, isum);
    } else {
        pt_span<DIM, 4, HB, T32>(a, R, sp.rep, sp.c_begin, sp.c_end, colour, sweep, thr, lane, nacc, nup, isum);
    }
    constexpr int Z = 2 * DIM;
    long long dP, dM;
    ising_deltas<Z>(nacc, nup, isum, dP, dM);
    long long v[3] = {dP, dM, (long long)nacc};
    unsigned long long* const dst[3] = {(unsigned long long*)&dcur[2 * sp.rep],
                                        (unsigned long long*)&dcur[2 * sp.rep + 1], &a.acc[sp.rep]};
    warp_add_atomic<3>(v, dst);
}

// One tile with its acceptance table `thr` (shared memory); per-warp atomics.
template <int DIM, bool HB, bool T32>
__device__ __forceinline__ void pt_run_tile(const PTArgs& a, const PTTile& tl, int colour,
                                            unsigned long long sweep, long long* dcur, const void* thr) {
    const PTReplica R = a.reps[tl.rep];
    int nacc = 0, nup = 0, isum = 0;
    if (R.V == 16) pt_tile<DIM, 16, HB, T32>(a, R, tl.rep, tl.c_begin, tl.c_end, colour, sweep, thr, nacc, nup, isum);
    else if (R.V == 8) pt_tile<DIM, 8, HB, T32>(a, R, tl.rep, tl.c_begin, tl.c_end, colour, sweep, thr, nacc, nup, isum);
    else pt_tile<DIM, 4, HB, T32>(a, R, tl.rep, tl.c_begin, tl.c_end, colour, sweep, thr, nacc, nup, isum);
    constexpr int Z = 2 * DIM;
    long long dP, dM;
    ising_deltas<Z>(nacc, nup, isum, dP, dM);
    long long v[3] = {dP, dM, (long long)nacc};
    unsigned long long* const dst[3] = {(unsigned long long*)&dcur[2 * tl.rep],
                                        (unsigned long long*)&dcur[2 * tl.rep + 1], &a.acc[tl.rep]};
    warp_add_atomic<3>(v, dst);
}

// log(U) of the exchange uniform of pair (p, p+1) of ladder l after sweep t
__device__ __forceinline__ double pt_exchange_logu(const PTArgs& a, int p, int l, unsigned long long t) {
    const uint4 w = philox10(make_uint4((uint32_t)p, (uint32_t)t, ctr_word2(t, 0, P_EXCHANGE), (uint32_t)l), a.k0, a.k1);
    return mcx_log(u53(w.x, w.y));
}

__device__ __forceinline__ bool pt_pair_active(const PTArgs& a, int gp, int stage, int& p, int& l) {
    p = a.pos_local[gp];
    l = a.pos_ladder[gp];
    const int first = (stage & 1) ? 1 : 0;
    return !(p < first || ((p - first) & 1) || p + 1 >= a.ladder_n[l]);
}

// The exchange step on block-local copies: pos (replica -> position), rep_at
// (global position -> replica), energies from (P, M).  Every thread handles the
// pairs whose lower global position it owns; pairs are disjoint, so the position
// updates never collide.  `count` adds the edge counters (done by one block only).
__device__ void pt_exchange(const PTArgs& a, int* s_pos, int* s_rep, const long long* s_P, const long long* s_M,
                            int stage, unsigned long long t, bool count, const double* logu) {
    for (int r = threadIdx.x; r < a.nrep; r += blockDim.x) s_rep[a.reps[r].gpos0 + s_pos[r]] = r;
    __syncthreads();
    for (int gp = threadIdx.x; gp < a.npos; gp += blockDim.x) {
        int p, l;
        if (!pt_pair_active(a, gp, stage, p, l)) continue;
        const int ri = s_rep[gp], rj = s_rep[gp + 1];
        const double lu = logu ? logu[gp] : pt_exchange_logu(a, p, l, t);
        const double bi = a.betas[gp], bj = a.betas[gp + 1];
        const double xi = (-(a.J * (double)s_P[ri])) - (a.h * (double)s_M[ri]);
        const double xj = (-(a.J * (double)s_P[rj])) - (a.h * (double)s_M[rj]);
        const double lr = (((-bi) * xj) - ((-bi) * xi)) + (((-bj) * xi) - ((-bj) * xj));
        const bool acc = (lr > 0.0) || (lu < lr);
        if (count) {
            a.ex_steps[gp] += 1ull;
            if (acc) a.ex_acc[gp] += 1ull;
        }
        if (acc) {
            s_pos[ri] = p + 1;
            s_pos[rj] = p;
        }
    }
    __syncthreads();
}

template <int DIM, bool HB, bool T32>
__global__ void __launch_bounds__(256, 2) k_pt_persistent(const PTArgs a) {
    extern __shared__ long long smem[];
    // [npos][16] tables (8 or 4 bytes per entry), then the per-replica state
    unsigned long long* s_tab = reinterpret_cast<unsigned long long*>(smem);
    uint32_t* s_tab32 = reinterpret_cast<uint32_t*>(smem);
    long long* s_P = smem + (size_t)a.npos * (T32 ? 8 : 16);
    long long* s_M = s_P + a.nrep;
    int* s_pos = reinterpret_cast<int*>(s_M + a.nrep);
    int* s_rep = s_pos + a.nrep;
    __shared__ unsigned s_gen;
    for (int i = threadIdx.x; i < a.npos * 16; i += blockDim.x) {
        if (T32) s_tab32[i] = a.tables32[i];
        else s_tab[i] = a.tables[i];
    }
    for (int r = threadIdx.x; r < a.nrep; r += blockDim.x) {
        s_P[r] = a.state[2 * r];
        s_M[r] = a.state[2 * r + 1];
        s_pos[r] = a.pos[r];
    }
    if (threadIdx.x == 0) s_gen = ld_acquire(&a.bar[1]);
    int stage = *a.stage;
    __syncthreads();
    unsigned gen = s_gen;
    const int lane = threadIdx.x & 31;
    const PTTile span = a.spans[blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)];  // this warp's share
    const size_t dsz = (size_t)a.nrep * 2;
    for (long long s = 0; s < a.nsweeps; ++s) {
        const unsigned long long t = a.sweep0 + (unsigned long long)s;
        long long* dcur = a.delta + (size_t)(s % 3) * dsz;
        const bool exch = (t + 1) % (unsigned long long)a.every == 0;
        double* logu = a.logu + (size_t)(s & 1) * a.npos;
        if (blockIdx.x == 0) {
            long long* dnext = a.delta + (size_t)((s + 1) % 3) * dsz;
            for (size_t i = threadIdx.x; i < dsz; i += blockDim.x) dnext[i] = 0;
        }
        if (exch)  // the exchange uniforms' logs, each computed once, read after the barriers
            for (int gp = blockIdx.x * blockDim.x + threadIdx.x; gp < a.npos; gp += gridDim.x * blockDim.x) {
                int p, l;
                if (pt_pair_active(a, gp, stage, p, l)) logu[gp] = pt_exchange_logu(a, p, l, t);
            }
        bool ok = true;
        for (int colour = 0; colour < 2; ++colour) {
            // every warp sweeps its own chunk range (static, balanced on the host), so
            // the phase needs no block barrier and no claiming
            if (span.c_end > span.c_begin && ok) {
                const int gpos = a.reps[span.rep].gpos0 + s_pos[span.rep];
                const void* tab = T32 ? (const void*)(s_tab32 + (size_t)gpos * 16) : (const void*)(s_tab + (size_t)gpos * 16);
                pt_run_span<DIM, HB, T32>(a, span, colour, t, dcur, tab, lane);
            }
            if (colour == 0) {
                // colour 1 of a replica needs only that replica's colour 0: its warps
                // count their arrivals (bounded wait; a timeout flags the error that
                // the grid barrier below reports)
                if (span.c_end > span.c_begin) {
                    __syncwarp();
                    if (lane == 0) {
                        __threadfence();
                        atomicAdd(&a.repbar[span.rep], 1ull);
                        const unsigned long long target = (unsigned long long)span.nw * (unsigned long long)(s + 1);
                        long long n = 0;
                        while (ld_acquire64(&a.repbar[span.rep]) < target) {
                            if (ld_acquire(&a.bar[2]) != 0u || ++n > a.spin_limit) {
                                atomicExch(&a.bar[2], 1u);
                                ok = false;
                                break;
                            }
                            __nanosleep(32);
                        }
                    }
                    ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
                }
            } else if (!grid_sync(a.bar, gridDim.x, gen, a.spin_limit)) {
                return;
            }
        }
        for (int r = threadIdx.x; r < a.nrep; r += blockDim.x) {
            s_P[r] += dcur[2 * r];
            s_M[r] += dcur[2 * r + 1];
        }
        __syncthreads();
        if (a.series && blockIdx.x == 0)
            for (int r = threadIdx.x; r < a.nrep; r += blockDim.x) {
                const int col = a.series_by_pos ? a.reps[r].gpos0 + s_pos[r] : r;
                a.series[((size_t)s * a.nrep + col) * 2] = s_P[r];
                a.series[((size_t)s * a.nrep + col) * 2 + 1] = s_M[r];
            }
        if (exch) {
            pt_exchange(a, s_pos, s_rep, s_P, s_M, stage, t, blockIdx.x == 0, logu);
            stage ^= 1;
        }
    }
    if (blockIdx.x == 0) {
        for (int r = threadIdx.x; r < a.nrep; r += blockDim.x) {
            a.pos[r] = s_pos[r];
            a.state[2 * r] = s_P[r];
            a.state[2 * r + 1] = s_M[r];
        }
        if (threadIdx.x == 0) *a.stage = stage;
    }
}

// Plain form: one launch per replica and colour (blocks = that replica's tiles).
template <int DIM, bool HB, bool T32>
__global__ void __launch_bounds__(256) k_pt_plain_half(const PTArgs a, int tile0, int colour,
                                                       unsigned long long sweep) {
    __shared__ unsigned long long s_thr[16];
    __shared__ uint32_t s_thr32[16];
    const PTTile tl = a.tiles[tile0 + blockIdx.x];
    if (threadIdx.x < 16) {
        const size_t e = (size_t)(a.reps[tl.rep].gpos0 + a.pos[tl.rep]) * 16 + threadIdx.x;
        if (T32) s_thr32[threadIdx.x] = a.tables32[e];
        else s_thr[threadIdx.x] = a.tables[e];
    }
    __syncthreads();
    pt_run_tile<DIM, HB, T32>(a, tl, colour, sweep, a.delta, T32 ? (const void*)s_thr32 : (const void*)s_thr);
}

// Plain form: fold the sweep's deltas into the state, record, exchange (one block).
__global__ void __launch_bounds__(256) k_pt_plain_exchange(const PTArgs a, long long s, unsigned long long t) {
    extern __shared__ long long smem[];
    long long* s_P = smem;
    long long* s_M = s_P + a.nrep;
    int* s_pos = reinterpret_cast<int*>(s_M + a.nrep);
    int* s_rep = s_pos + a.nrep;
    for (int r = threadIdx.x; r < a.nrep; r += blockDim.x) {
        s_P[r] = a.state[2 * r] + a.delta[2 * r];
        s_M[r] = a.state[2 * r + 1] + a.delta[2 * r + 1];
        a.delta[2 * r] = 0;
        a.delta[2 * r + 1] = 0;
        a.state[2 * r] = s_P[r];
        a.state[2 * r + 1] = s_M[r];
        s_pos[r] = a.pos[r];
        if (a.series) {
            const int col = a.series_by_pos ? a.reps[r].gpos0 + s_pos[r] : r;
            a.series[((size_t)s * a.nrep + col) * 2] = s_P[r];
            a.series[((size_t)s * a.nrep + col) * 2 + 1] = s_M[r];
        }
    }
    __syncthreads();
    if ((t + 1) % (unsigned long long)a.every != 0) return;
    const int stage = *a.stage;
    pt_exchange(a, s_pos, s_rep, s_P, s_M, stage, t, true, nullptr);
    for (int r = threadIdx.x; r < a.nrep; r += blockDim.x) a.pos[r] = s_pos[r];
    if (threadIdx.x == 0) *a.stage = stage ^ 1;
}

// Bounded wait on a flag nothing sets: the failure-detection path of the barriers,
// testable without faulting or hanging the GPU.
__global__ void k_wait_flag(unsigned* flag, long long limit, unsigned* result) {
    long long n = 0;
    while (ld_acquire(flag) == 0u) {
        if (++n > limit) {
            *result = 1u;
            return;
        }
        __nanosleep(100);
    }
    *result = 0u;
}

}  // namespace mcx

using namespace mcx;

struct mcx_pt {
    mcx_ctx* ctx = nullptr;
    mcx::CtxHold hold;  // keeps ctx alive while this object exists
    int dim = 3;
    double J = 1, h = 0;
    int nladders = 0, nrep = 0, npos = 0;
    std::vector<int> ladder_n, ladder_side, ladder_gpos0, rep_ladder;
    std::vector<double> betas;
    std::vector<PTReplica> reps;
    std::vector<PTTile> tiles;
    std::vector<int> rep_tile0, rep_ntiles;
    int64_t sites = 0;
    size_t arena_bytes = 0;
    int8_t* d_arena = nullptr;
    PTReplica* d_reps = nullptr;
    PTTile* d_tiles = nullptr;
    PTTile* d_spans = nullptr;       // [grid * 8] warp chunk ranges of the persistent form
    int grid = 0;                    // persistent grid size
    unsigned long long* d_tables = nullptr;  // [3 algs][npos][16]
    uint32_t* d_tables32 = nullptr;          // [3 algs][npos][16], entry - 1
    bool fits32[3] = {false, false, false};  // every entry of the algorithm's tables >= 1
    double* d_betas = nullptr;
    int* d_pos_ladder = nullptr;
    int* d_pos_local = nullptr;
    int* d_ladder_n = nullptr;
    int32_t* d_pos = nullptr;
    int32_t* d_stage = nullptr;
    long long* d_state = nullptr;
    long long* d_delta = nullptr;
    unsigned long long* d_acc = nullptr;
    unsigned long long* d_ex_steps = nullptr;
    unsigned long long* d_ex_acc = nullptr;
    long long* d_series = nullptr;
    int64_t series_cap = 0;
    int record = 0;                // 0: series on request, by replica; 1: always, by replica;
                                   // 2: always, by ladder position
    int64_t series_len = 0;        // sweeps the device series holds (last run)
    int series_by_pos = 0;
    unsigned int* d_bar = nullptr;
    unsigned long long* d_repbar = nullptr;  // [nrep] per-replica arrival counters (persistent form)
    double* d_logu = nullptr;
    int8_t* d_lin = nullptr;
    size_t lin_bytes = 0;
    std::vector<std::pair<void*, size_t>> allocs;
    long long spin_limit = 1ll << 24;
    // schedule of the persistent form (results never depend on it)
    int bps_max = 1;       // co-resident blocks per SM of the persistent kernel
    int sched_bps = 1;     // blocks per SM in use
    int sched_vcap = 16;   // widest chunk (sites per thread) a replica may use
    int sched_weights = 0; // cost weights of the warp split (0, 1, 2)
};

namespace mcx {

static uint32_t roundup_recip(uint32_t d) { return d <= 1 ? 0u : (uint32_t)(((1ull << 32) + d - 1) / d); }

static mcx_status pt_alloc(mcx_pt* pt, void** p, size_t bytes) {
    MCX_CHECK(dev_alloc(pt->ctx, p, bytes));
    pt->allocs.emplace_back(*p, bytes);
    return MCX_OK;
}

template <typename T>
static mcx_status pt_upload(mcx_pt* pt, T** dst, const std::vector<T>& v) {
    void* p = nullptr;
    MCX_CHECK(pt_alloc(pt, &p, std::max<size_t>(1, v.size()) * sizeof(T)));
    if (!v.empty()) MCX_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    *dst = (T*)p;
    return MCX_OK;
}

// Replaces the device copy held in *dst (allocated by pt_upload) by a new upload of v.
template <typename T>
static mcx_status pt_reupload(mcx_pt* pt, T** dst, const std::vector<T>& v) {
    for (auto it = pt->allocs.begin(); it != pt->allocs.end(); ++it)
        if (it->first == (void*)*dst) {
            dev_free(pt->ctx, it->first, it->second);
            pt->allocs.erase(it);
            break;
        }
    *dst = nullptr;
    return pt_upload(pt, dst, v);
}

using PersistentFn = void (*)(const PTArgs);
using PlainFn = void (*)(const PTArgs, int, int, unsigned long long);

template <int DIM, bool T32>
static PersistentFn persistent_fn_t(bool hb) {
    return hb ? k_pt_persistent<DIM, true, T32> : k_pt_persistent<DIM, false, T32>;
}

static PersistentFn persistent_fn(int dim, bool hb, bool t32) {
    if (dim == 2) return t32 ? persistent_fn_t<2, true>(hb) : persistent_fn_t<2, false>(hb);
    return t32 ? persistent_fn_t<3, true>(hb) : persistent_fn_t<3, false>(hb);
}

template <int DIM, bool T32>
static PlainFn plain_fn_t(bool hb) {
    return hb ? k_pt_plain_half<DIM, true, T32> : k_pt_plain_half<DIM, false, T32>;
}

static PlainFn plain_fn(int dim, bool hb, bool t32) {
    if (dim == 2) return t32 ? plain_fn_t<2, true>(hb) : plain_fn_t<2, false>(hb);
    return t32 ? plain_fn_t<3, true>(hb) : plain_fn_t<3, false>(hb);
}

static size_t pt_smem(const mcx_pt* pt) {
    return (size_t)pt->nrep * (2 * sizeof(long long) + sizeof(int)) + (size_t)pt->npos * sizeof(int);
}

static size_t pt_smem_persistent(const mcx_pt* pt, bool t32) {
    return pt_smem(pt) + (size_t)pt->npos * 16 * (t32 ? 4 : 8);
}

// Warp spans of the persistent form: every warp of the grid sweeps one chunk range of
// one replica per phase.  Replica r gets k_r warps, handed out one at a time to the
// replica whose cost per warp is largest (costs per site: 1.0 for 16-site rows chunks,
// 1.15 for 8, 1.4 for 4), and its chunks are split evenly among them.
// 3-D ladders: the units are (replica, plane column): chunks [32j, 32j + 32) of every plane
// (fewer in a plane's last column), each walked through the planes by its warps (pt_zwalk).
// A warp's time per plane does not depend on how many of its lanes have a chunk, so a unit
// costs Lz planes at the per-chunk weight of its width; unit u gets k_u warps (the next warp
// to the largest cost per warp, at most one plane each), which split its planes evenly.
// Returns false (nothing changed) when there are more units than warps.
static bool pt_schedule_planes(mcx_pt* pt, int nwarps, const double* w, std::vector<PTTile>& spans) {
    struct Unit {
        int r, c0, c1;
        double cost;
    };
    std::vector<Unit> units;
    for (int r = 0; r < pt->nrep; ++r) {
        const PTReplica& P = pt->reps[r];
        const int pc = P.cpr * P.Ly;
        const double c = (double)P.Lz * P.V * (P.V == 16 ? w[0] : (P.V == 8 ? w[1] : w[2]));
        for (int c0 = 0; c0 < pc; c0 += 32) units.push_back(Unit{r, c0, std::min(pc, c0 + 32), c});
    }
    const int U = (int)units.size();
    if (U > nwarps) return false;
    std::vector<int> k(U, 1), kr(pt->nrep, 0);
    std::priority_queue<std::pair<double, int>> heap;
    for (int u = 0; u < U; ++u) heap.push({units[u].cost, u});
    for (int left = nwarps - U; left > 0 && !heap.empty();) {
        const int u = heap.top().second;
        heap.pop();
        if (k[u] >= pt->reps[units[u].r].Lz) continue;  // one plane per warp at most
        ++k[u];
        --left;
        heap.push({units[u].cost / k[u], u});
    }
    for (int u = 0; u < U; ++u) kr[units[u].r] += k[u];
    spans.clear();
    for (int u = 0; u < U; ++u) {
        const PTReplica& P = pt->reps[units[u].r];
        for (int j = 0; j < k[u]; ++j) {
            PTTile t;
            std::memset(&t, 0, sizeof(t));
            t.rep = units[u].r;
            t.c_begin = units[u].c0;
            t.c_end = units[u].c1;
            t.zb = (int)((long long)j * P.Lz / k[u]);
            t.ze = (int)((long long)(j + 1) * P.Lz / k[u]);
            t.sites = (t.c_end - t.c_begin) * P.V * (t.ze - t.zb);
            t.nw = kr[units[u].r];
            spans.push_back(t);
        }
    }
    return true;
}

static mcx_status pt_schedule(mcx_pt* pt, int grid, int weights) {
    static const double kW[3][3] = {{1.0, 1.15, 1.4}, {1.0, 1.0, 1.0}, {1.0, 1.3, 1.8}};
    const double* w = kW[weights];
    const int nwarps = grid * 8;
    const int R = pt->nrep;
    if (pt->dim == 3) {
        std::vector<PTTile> spans;
        if (pt_schedule_planes(pt, nwarps, w, spans)) {
            PTTile idle;
            std::memset(&idle, 0, sizeof(idle));
            spans.resize(nwarps, idle);
            MCX_CHECK(pt_reupload(pt, &pt->d_spans, spans));
            pt->grid = grid;
            return MCX_OK;
        }
    }
    if (nwarps < R) return fail(MCX_ERR_INVALID_ARG, "%d replicas need at least as many resident warps", R);
    std::vector<double> cost(R);
    std::vector<int> nch(R), k(R, 1);
    std::priority_queue<std::pair<double, int>> heap;
    for (int r = 0; r < R; ++r) {
        const PTReplica& P = pt->reps[r];
        nch[r] = P.cpr * P.rows;
        cost[r] = (double)nch[r] * P.V * (P.V == 16 ? w[0] : (P.V == 8 ? w[1] : w[2]));
        heap.push({cost[r], r});
    }
    for (int left = nwarps - R; left > 0 && !heap.empty();) {
        const int r = heap.top().second;
        heap.pop();
        if (k[r] >= nch[r]) continue;  // one chunk per warp at most
        ++k[r];
        --left;
        heap.push({cost[r] / k[r], r});
    }
    std::vector<PTTile> spans;
    spans.reserve(nwarps);
    for (int r = 0; r < R; ++r)
        for (int j = 0; j < k[r]; ++j) {
            PTTile t;
            std::memset(&t, 0, sizeof(t));  // zb = ze = 0: a chunk range
            t.rep = r;
            t.c_begin = (int)((long long)j * nch[r] / k[r]);
            t.c_end = (int)((long long)(j + 1) * nch[r] / k[r]);
            t.sites = (t.c_end - t.c_begin) * pt->reps[r].V;
            t.nw = k[r];
            spans.push_back(t);
        }
    PTTile idle;
    std::memset(&idle, 0, sizeof(idle));
    spans.resize(nwarps, idle);
    MCX_CHECK(pt_reupload(pt, &pt->d_spans, spans));
    pt->grid = grid;
    return MCX_OK;
}

// Sites per thread of every replica: the widest of 16, 8, 4 that divides its colour rows and is
// at most vcap (rows of a multiple of 4 sites always admit 4); the plain form's tiles of about
// 4096 same-colour sites follow.  The random stream does not depend on the width.
static mcx_status pt_set_widths(mcx_pt* pt, int vcap) {
    pt->tiles.clear();
    pt->rep_tile0.clear();
    pt->rep_ntiles.clear();
    for (int r = 0; r < pt->nrep; ++r) {
        PTReplica& R = pt->reps[r];
        R.V = (R.W % 16 == 0 && vcap >= 16) ? 16 : ((R.W % 8 == 0 && vcap >= 8) ? 8 : 4);
        R.cpr = R.W / R.V;
        R.m_cpr = roundup_recip((uint32_t)R.cpr);
        const int nchunks = R.cpr * R.rows;
        const int per = 256 * (16 / R.V);
        pt->rep_tile0.push_back((int)pt->tiles.size());
        for (int c = 0; c < nchunks; c += per) {
            PTTile t;
            std::memset(&t, 0, sizeof(t));
            t.rep = r;
            t.c_begin = c;
            t.c_end = std::min(nchunks, c + per);
            t.sites = (t.c_end - t.c_begin) * R.V;
            pt->tiles.push_back(t);
        }
        pt->rep_ntiles.push_back((int)pt->tiles.size() - pt->rep_tile0.back());
    }
    MCX_CHECK(pt_reupload(pt, &pt->d_reps, pt->reps));
    MCX_CHECK(pt_reupload(pt, &pt->d_tiles, pt->tiles));
    return MCX_OK;
}

// Applies a schedule (validated by the caller).
static mcx_status pt_apply_schedule(mcx_pt* pt, int bps, int vcap, int weights) {
    MCX_CUDA(cudaStreamSynchronize(pt->ctx->stream));  // no launch may read the old descriptors
    if (vcap != pt->sched_vcap) MCX_CHECK(pt_set_widths(pt, vcap));
    MCX_CHECK(pt_schedule(pt, pt->ctx->num_sms * bps, weights));
    pt->sched_bps = bps;
    pt->sched_vcap = vcap;
    pt->sched_weights = weights;
    return MCX_OK;
}

static void pt_args(const mcx_pt* pt, PTArgs* a, mcx_algorithm alg) {
    std::memset(a, 0, sizeof(*a));
    a->arena = pt->d_arena;
    a->reps = pt->d_reps;
    a->tiles = pt->d_tiles;
    a->spans = pt->d_spans;
    a->nrep = pt->nrep;
    a->ntiles = (int)pt->tiles.size();
    a->npos = pt->npos;
    a->tables = pt->d_tables + (size_t)alg * pt->npos * 16;
    a->tables32 = pt->d_tables32 + (size_t)alg * pt->npos * 16;
    a->betas = pt->d_betas;
    a->pos_ladder = pt->d_pos_ladder;
    a->pos_local = pt->d_pos_local;
    a->ladder_n = pt->d_ladder_n;
    a->pos = pt->d_pos;
    a->stage = pt->d_stage;
    a->state = pt->d_state;
    a->delta = pt->d_delta;
    a->acc = pt->d_acc;
    a->ex_steps = pt->d_ex_steps;
    a->ex_acc = pt->d_ex_acc;
    a->bar = pt->d_bar;
    a->repbar = pt->d_repbar;
    a->logu = pt->d_logu;
    a->J = pt->J;
    a->h = pt->h;
    a->series_by_pos = 0;
    a->spin_limit = pt->spin_limit;
}

// colour-split layout conversion for one replica (reuses the lattice kernels' rule)
__global__ void k_pt_scatter(int8_t* __restrict__ lin, int8_t* __restrict__ c0, int8_t* __restrict__ c1,
                             int Lx, int Ly, int Lz, int W, int to_device) {
    const long long N = (long long)Lx * Ly * Lz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % Lx);
        const long long rr = i / Lx;
        const int y = (int)(rr % Ly), z = (int)(rr / Ly);
        const long long e = (long long)(y + Ly * z) * W + (x >> 1);
        int8_t* col = ((x + y + z) & 1) ? c1 : c0;
        if (to_device) col[e] = lin[i];
        else lin[i] = col[e];
    }
}

__global__ void k_pt_init_random(int8_t* arena, const PTReplica* reps, int nrep, uint32_t k0, uint32_t k1) {
    const int r = blockIdx.y;
    if (r >= nrep) return;
    const PTReplica R = reps[r];
    const int Lx = 2 * R.W;
    const long long N = (long long)Lx * R.rows;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % Lx);
        const long long rr = i / Lx;
        const int y = (int)(rr % R.Ly), z = (int)(rr / R.Ly);
        const int c = (x + y + z) & 1;
        const uint4 w = philox10(make_uint4((uint32_t)(i >> 3), 0u, ctr_word2(0ull, c, P_INIT), (uint32_t)r), k0, k1);
        const uint32_t u = pick4(w, (int)((i >> 1) & 3));
        arena[R.off[c] + rr * R.W + (x >> 1)] = (int8_t)((u & 0x80000000u) ? 1 : -1);
    }
}

// per-replica (pair_sum, spin_sum) recompute
__global__ void k_pt_observables(const int8_t* arena, const PTReplica* reps, int nrep, int dim, long long* state) {
    const int r = blockIdx.y;
    if (r >= nrep) return;
    const PTReplica R = reps[r];
    const int8_t* c0 = arena + R.off[0];
    const int8_t* c1 = arena + R.off[1];
    long long P = 0, M = 0;
    const long long half = (long long)R.W * R.rows;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < half;
         e += (long long)gridDim.x * blockDim.x) {
        const int row = (int)(e / R.W), k = (int)(e - (long long)row * R.W);
        const int y = row % R.Ly, z = row / R.Ly;
        const int p = (y + z) & 1;
        const int s = c0[e];
        const int km = k == 0 ? R.W - 1 : k - 1, kp = k == R.W - 1 ? 0 : k + 1;
        const long long rb = (long long)row * R.W;
        int S = c1[rb + k] + c1[rb + (p ? kp : km)];
        const int yp = y + 1 == R.Ly ? 0 : y + 1, ym = y == 0 ? R.Ly - 1 : y - 1;
        S += c1[(long long)(yp + R.Ly * z) * R.W + k] + c1[(long long)(ym + R.Ly * z) * R.W + k];
        if (dim == 3) {
            const int zp = z + 1 == R.Lz ? 0 : z + 1, zm = z == 0 ? R.Lz - 1 : z - 1;
            S += c1[(long long)(y + R.Ly * zp) * R.W + k] + c1[(long long)(y + R.Ly * zm) * R.W + k];
        }
        P += s * S;
        M += s + c1[e];
    }
    long long v[2] = {P, M};
    unsigned long long* const dst[2] = {(unsigned long long*)&state[2 * r], (unsigned long long*)&state[2 * r + 1]};
    block_add_atomic<2>(v, dst);
}

static mcx_status pt_recompute(mcx_pt* pt) {
    mcx_ctx* ctx = pt->ctx;
    MCX_CUDA(cudaMemsetAsync(pt->d_state, 0, (size_t)pt->nrep * 2 * sizeof(long long), ctx->stream));
    dim3 grid(8, pt->nrep);
    k_pt_observables<<<grid, 256, 0, ctx->stream>>>(pt->d_arena, pt->d_reps, pt->nrep, pt->dim, pt->d_state);
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

}  // namespace mcx

extern "C" {

MCX_API mcx_status mcx_pt_destroy(mcx_pt* pt) {
    if (!pt) return MCX_OK;
    cudaStreamSynchronize(pt->ctx->stream);
    for (auto& a : pt->allocs) dev_free(pt->ctx, a.first, a.second);
    delete pt;
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_create(mcx_ctx* ctx, int dim, int nladders, const int32_t* sides,
                                 const int32_t* nreplicas, const double* betas, double J, double h,
                                 mcx_pt** out) {
    if (!ctx || !sides || !nreplicas || !betas || !out) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (dim != 2 && dim != 3) return fail(MCX_ERR_INVALID_ARG, "dim must be 2 or 3");
    if (nladders < 1) return fail(MCX_ERR_INVALID_ARG, "need at least one ladder");
    if (!std::isfinite(J) || !std::isfinite(h)) return fail(MCX_ERR_INVALID_ARG, "J and h must be finite");
    mcx_pt* pt = new mcx_pt();
    pt->ctx = ctx;
    pt->hold.set(ctx);
    pt->dim = dim;
    pt->J = J;
    pt->h = h;
    pt->nladders = nladders;
    std::vector<int> pos_ladder, pos_local;
    for (int l = 0; l < nladders; ++l) {
        const int L = sides[l], n = nreplicas[l];
        if (n < 2) {
            delete pt;
            return fail(MCX_ERR_INVALID_ARG, "ladder %d: need at least 2 replicas", l);
        }
        if (L < 8 || L % 8) {
            delete pt;
            return fail(MCX_ERR_INVALID_ARG, "ladder %d: side %d must be a multiple of 8", l, L);
        }
        pt->ladder_n.push_back(n);
        pt->ladder_side.push_back(L);
        pt->ladder_gpos0.push_back(pt->npos);
        for (int p = 0; p < n; ++p) {
            const double b = betas[pt->npos + p];
            if (!std::isfinite(b)) {
                delete pt;
                return fail(MCX_ERR_INVALID_ARG, "beta must be finite");
            }
            pt->betas.push_back(b);
            pos_ladder.push_back(l);
            pos_local.push_back(p);
            pt->rep_ladder.push_back(l);
        }
        pt->npos += n;
    }
    pt->nrep = pt->npos;
    if (pt->nrep > 1024) {
        delete pt;
        return fail(MCX_ERR_INVALID_ARG, "at most 1024 replicas");
    }
    // arena layout: replica r (ladder order), colour 0 then colour 1, 256-byte aligned
    size_t off = 0;
    for (int r = 0; r < pt->nrep; ++r) {
        const int l = pt->rep_ladder[r];
        const int L = pt->ladder_side[l];
        PTReplica R;
        std::memset(&R, 0, sizeof(R));
        R.W = L / 2;
        R.Ly = L;
        R.Lz = dim == 3 ? L : 1;
        R.rows = R.Ly * R.Lz;
        R.V = R.W % 16 == 0 ? 16 : (R.W % 8 == 0 ? 8 : 4);
        R.cpr = R.W / R.V;
        R.ladder = l;
        R.gpos0 = pt->ladder_gpos0[l];
        R.n = pt->ladder_n[l];
        R.m_cpr = roundup_recip((uint32_t)R.cpr);
        R.m_Ly = roundup_recip((uint32_t)R.Ly);
        const size_t half = (size_t)R.W * R.rows;
        R.off[0] = (long long)off;
        off += (half + 255) / 256 * 256;
        R.off[1] = (long long)off;
        off += (half + 255) / 256 * 256;
        pt->sites += 2 * (int64_t)half;
        pt->lin_bytes = std::max(pt->lin_bytes, 2 * half);
        pt->reps.push_back(R);
        // tiles of ~4096 same-colour sites
        const int nchunks = R.cpr * R.rows;
        const int per = 256 * (16 / R.V);
        pt->rep_tile0.push_back((int)pt->tiles.size());
        for (int c = 0; c < nchunks; c += per) {
            PTTile t;
            std::memset(&t, 0, sizeof(t));
            t.rep = r;
            t.c_begin = c;
            t.c_end = std::min(nchunks, c + per);
            t.sites = (t.c_end - t.c_begin) * R.V;
            pt->tiles.push_back(t);
        }
        pt->rep_ntiles.push_back((int)pt->tiles.size() - pt->rep_tile0.back());
    }
    pt->arena_bytes = off;
    mcx_status st = MCX_OK;
    auto run = [&](mcx_status s) {
        if (st == MCX_OK) st = s;
    };
    void* p = nullptr;
    run(pt_alloc(pt, &p, pt->arena_bytes));
    pt->d_arena = (int8_t*)p;
    run(pt_upload(pt, &pt->d_reps, pt->reps));
    run(pt_upload(pt, &pt->d_tiles, pt->tiles));
    run(pt_upload(pt, &pt->d_betas, pt->betas));
    run(pt_upload(pt, &pt->d_pos_ladder, pos_ladder));
    run(pt_upload(pt, &pt->d_pos_local, pos_local));
    run(pt_upload(pt, &pt->d_ladder_n, pt->ladder_n));
    // acceptance tables for the three algorithms at every ladder position
    std::vector<unsigned long long> tabs((size_t)3 * pt->npos * 16, 0);
    for (int alg = 0; alg < 3 && st == MCX_OK; ++alg)
        for (int gp = 0; gp < pt->npos; ++gp) {
            Table t;
            run(build_ising_table(dim, (mcx_algorithm)alg, pt->betas[gp], J, h, &t));
            for (int i = 0; i < t.n; ++i)
                tabs[((size_t)alg * pt->npos + gp) * 16 + i] =
                    ising_tab_entry(t.thr[i], i, 2 * dim, alg == MCX_HEATBATH);
        }
    run(pt_upload(pt, &pt->d_tables, tabs));
    std::vector<uint32_t> tabs32(tabs.size());
    for (int alg = 0; alg < 3; ++alg) {
        pt->fits32[alg] = true;
        for (int gp = 0; gp < pt->npos; ++gp)
            for (int i = 0; i < 16; ++i) {
                const size_t e = ((size_t)alg * pt->npos + gp) * 16 + i;
                if (i < 2 * (2 * dim + 1) && tabs[e] == 0) pt->fits32[alg] = false;
                tabs32[e] = (uint32_t)(tabs[e] - 1);
            }
    }
    run(pt_upload(pt, &pt->d_tables32, tabs32));
    std::vector<int32_t> pos0(pt->nrep);
    for (int r = 0; r < pt->nrep; ++r) pos0[r] = r - pt->ladder_gpos0[pt->rep_ladder[r]];
    run(pt_upload(pt, &pt->d_pos, pos0));
    run(pt_upload(pt, &pt->d_stage, std::vector<int32_t>(1, 0)));
    run(pt_upload(pt, &pt->d_state, std::vector<long long>((size_t)pt->nrep * 2, 0)));
    run(pt_upload(pt, &pt->d_delta, std::vector<long long>((size_t)pt->nrep * 6, 0)));
    run(pt_upload(pt, &pt->d_acc, std::vector<unsigned long long>(pt->nrep, 0)));
    run(pt_upload(pt, &pt->d_ex_steps, std::vector<unsigned long long>(pt->npos, 0)));
    run(pt_upload(pt, &pt->d_ex_acc, std::vector<unsigned long long>(pt->npos, 0)));
    run(pt_upload(pt, &pt->d_bar, std::vector<unsigned int>(4, 0)));
    run(pt_upload(pt, &pt->d_repbar, std::vector<unsigned long long>(pt->nrep, 0ull)));
    run(pt_upload(pt, &pt->d_logu, std::vector<double>((size_t)2 * pt->npos, 0.0)));
    run(pt_alloc(pt, &p, pt->lin_bytes));
    pt->d_lin = (int8_t*)p;
    if (st == MCX_OK) {
        // schedule for the persistent grid
        // one grid for every variant: the smallest co-resident block count among them
        int bps = 1 << 30;
        for (int v = 0; v < 4; ++v) {
            const bool hb = v & 1, t32 = v >> 1;
            const size_t smem = pt_smem_persistent(pt, t32);
            const PersistentFn fn = persistent_fn(dim, hb, t32);
            cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            int b = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, 256, smem) != cudaSuccess || b < 1) b = 1;
            bps = std::min(bps, b);
        }
        cudaFuncSetAttribute(k_pt_plain_exchange, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pt_smem(pt));
        pt->bps_max = bps;
        pt->sched_bps = bps;
        run(pt_schedule(pt, ctx->num_sms * bps, 0));
    }
    if (st == MCX_OK) {
        // all spins up, like the reference constructors
        MCX_CUDA(cudaMemset(pt->d_arena, 1, pt->arena_bytes));
        run(pt_recompute(pt));
    }
    if (st != MCX_OK) {
        mcx_pt_destroy(pt);
        return st;
    }
    *out = pt;
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_info(const mcx_pt* pt, int32_t* nreplicas, int64_t* sites, int64_t* device_bytes) {
    if (!pt) return fail(MCX_ERR_INVALID_ARG, "pt is NULL");
    if (nreplicas) *nreplicas = pt->nrep;
    if (sites) *sites = pt->sites;
    if (device_bytes) {
        int64_t b = 0;
        for (auto& a : pt->allocs) b += (int64_t)a.second;
        *device_bytes = b;
    }
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_init_random(mcx_pt* pt, uint64_t seed) {
    if (!pt) return fail(MCX_ERR_INVALID_ARG, "pt is NULL");
    mcx_ctx* ctx = pt->ctx;
    dim3 grid(16, pt->nrep);
    k_pt_init_random<<<grid, 256, 0, ctx->stream>>>(pt->d_arena, pt->d_reps, pt->nrep, (uint32_t)seed,
                                                     (uint32_t)(seed >> 32));
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    return pt_recompute(pt);
}

static mcx_status pt_copy_spins(mcx_pt* pt, int32_t r, int8_t* host, size_t n, bool to_device) {
    if (!pt || !host) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (r < 0 || r >= pt->nrep) return fail(MCX_ERR_INVALID_ARG, "replica %d out of range", r);
    const PTReplica& R = pt->reps[r];
    const size_t N = (size_t)2 * R.W * R.rows;
    if (n != N) return fail(MCX_ERR_INVALID_ARG, "replica %d has %zu sites, got %zu", r, N, n);
    mcx_ctx* ctx = pt->ctx;
    if (to_device) {
        for (size_t i = 0; i < n; ++i)
            if (host[i] != 1 && host[i] != -1) return fail(MCX_ERR_INVALID_ARG, "spin %zu is %d", i, (int)host[i]);
        MCX_CUDA(cudaMemcpyAsync(pt->d_lin, host, n, cudaMemcpyHostToDevice, ctx->stream));
    }
    k_pt_scatter<<<64, 256, 0, ctx->stream>>>(pt->d_lin, pt->d_arena + R.off[0], pt->d_arena + R.off[1], 2 * R.W,
                                              R.Ly, R.Lz, R.W, to_device ? 1 : 0);
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    if (to_device) return pt_recompute(pt);
    MCX_CUDA(cudaMemcpyAsync(host, pt->d_lin, n, cudaMemcpyDeviceToHost, ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_set_spins(mcx_pt* pt, int32_t replica, const int8_t* host, size_t n) {
    return pt_copy_spins(pt, replica, const_cast<int8_t*>(host), n, true);
}

MCX_API mcx_status mcx_pt_get_spins(mcx_pt* pt, int32_t replica, int8_t* host, size_t n) {
    return pt_copy_spins(pt, replica, host, n, false);
}

MCX_API mcx_status mcx_pt_run(mcx_pt* pt, mcx_algorithm alg, mcx_rng* rng, int64_t nsweeps,
                              int32_t exchange_every, mcx_pt_mode mode, int64_t* series) {
    if (!pt || !rng) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (alg != MCX_METROPOLIS && alg != MCX_GLAUBER && alg != MCX_HEATBATH)
        return fail(MCX_ERR_INVALID_ARG, "unknown algorithm");
    if (nsweeps < 0 || exchange_every < 1) return fail(MCX_ERR_INVALID_ARG, "nsweeps >= 0 and exchange_every >= 1");
    if (mode != MCX_PT_PERSISTENT && mode != MCX_PT_PLAIN) return fail(MCX_ERR_INVALID_ARG, "unknown mode");
    if (rng->counter + (uint64_t)nsweeps >= (1ull << 48)) return fail(MCX_ERR_INVALID_ARG, "sweep counter beyond 2^48");
    if (nsweeps == 0) return MCX_OK;
    mcx_ctx* ctx = pt->ctx;
    const bool rec = series != nullptr || pt->record != 0;
    if (rec) {
        if (nsweeps > pt->series_cap) {
            void* p = nullptr;
            MCX_CHECK(dev_alloc(ctx, &p, (size_t)nsweeps * pt->nrep * 2 * sizeof(long long)));
            for (auto it = pt->allocs.begin(); it != pt->allocs.end(); ++it)
                if (it->first == pt->d_series) {
                    dev_free(ctx, it->first, it->second);
                    pt->allocs.erase(it);
                    break;
                }
            pt->allocs.emplace_back(p, (size_t)nsweeps * pt->nrep * 2 * sizeof(long long));
            pt->d_series = (long long*)p;
            pt->series_cap = nsweeps;
        }
    }
    PTArgs a;
    pt_args(pt, &a, alg);
    a.series = rec ? pt->d_series : nullptr;
    a.series_by_pos = pt->record == 2 ? 1 : 0;
    a.k0 = (uint32_t)rng->seed;
    a.k1 = (uint32_t)(rng->seed >> 32);
    a.sweep0 = rng->counter;
    a.nsweeps = nsweeps;
    a.every = exchange_every;
    const bool hb = alg == MCX_HEATBATH;
    const bool t32 = pt->fits32[alg];
    const size_t smem = pt_smem(pt);
    const size_t smem_persistent = pt_smem_persistent(pt, t32);
    MCX_CUDA(cudaMemsetAsync(pt->d_acc, 0, (size_t)pt->nrep * sizeof(unsigned long long), ctx->stream));
    if (mode == MCX_PT_PERSISTENT) {
        MCX_CUDA(cudaMemsetAsync(pt->d_delta, 0, (size_t)pt->nrep * 6 * sizeof(long long), ctx->stream));
        MCX_CUDA(cudaMemsetAsync(pt->d_bar, 0, sizeof(unsigned int), ctx->stream));
        MCX_CUDA(cudaMemsetAsync(pt->d_bar + 2, 0, sizeof(unsigned int), ctx->stream));
        MCX_CUDA(cudaMemsetAsync(pt->d_repbar, 0, (size_t)pt->nrep * sizeof(unsigned long long), ctx->stream));
        const PersistentFn fn = persistent_fn(pt->dim, hb, t32);
        void* args[] = {&a};
        MCX_CUDA(cudaLaunchCooperativeKernel((const void*)fn, dim3(pt->grid), dim3(256), args, smem_persistent,
                                             ctx->stream));
        count_launch(ctx);
        unsigned int err = 0;
        MCX_CUDA(cudaMemcpyAsync(&err, pt->d_bar + 2, sizeof(err), cudaMemcpyDeviceToHost, ctx->stream));
        MCX_CUDA(cudaStreamSynchronize(ctx->stream));
        if (err) return fail(MCX_ERR_TIMEOUT, "grid barrier wait exceeded its limit");
    } else {
        MCX_CUDA(cudaMemsetAsync(pt->d_delta, 0, (size_t)pt->nrep * 2 * sizeof(long long), ctx->stream));
        const PlainFn fn = plain_fn(pt->dim, hb, t32);
        for (int64_t s = 0; s < nsweeps; ++s) {
            const unsigned long long t = rng->counter + (unsigned long long)s;
            for (int r = 0; r < pt->nrep; ++r)
                for (int c = 0; c < 2; ++c)
                    fn<<<pt->rep_ntiles[r], 256, 0, ctx->stream>>>(a, pt->rep_tile0[r], c, t);
            k_pt_plain_exchange<<<1, 256, smem, ctx->stream>>>(a, s, t);
        }
        count_launch(ctx, (uint64_t)nsweeps * (2 * pt->nrep + 1));
        MCX_CUDA(cudaGetLastError());
    }
    rng->counter += (uint64_t)nsweeps;
    pt->series_len = rec ? nsweeps : 0;
    pt->series_by_pos = a.series_by_pos;
    if (series) {
        MCX_CUDA(cudaMemcpyAsync(series, pt->d_series, (size_t)nsweeps * pt->nrep * 2 * sizeof(long long),
                                 cudaMemcpyDeviceToHost, ctx->stream));
        MCX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_indices(mcx_pt* pt, int32_t* pos, int32_t* stage) {
    if (!pt) return fail(MCX_ERR_INVALID_ARG, "pt is NULL");
    if (pos) MCX_CUDA(cudaMemcpyAsync(pos, pt->d_pos, pt->nrep * sizeof(int32_t), cudaMemcpyDeviceToHost, pt->ctx->stream));
    if (stage) MCX_CUDA(cudaMemcpyAsync(stage, pt->d_stage, sizeof(int32_t), cudaMemcpyDeviceToHost, pt->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(pt->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_exchange_counters(mcx_pt* pt, uint64_t* steps, uint64_t* accepted) {
    if (!pt) return fail(MCX_ERR_INVALID_ARG, "pt is NULL");
    std::vector<unsigned long long> s(pt->npos), a(pt->npos);
    MCX_CUDA(cudaMemcpyAsync(s.data(), pt->d_ex_steps, pt->npos * 8, cudaMemcpyDeviceToHost, pt->ctx->stream));
    MCX_CUDA(cudaMemcpyAsync(a.data(), pt->d_ex_acc, pt->npos * 8, cudaMemcpyDeviceToHost, pt->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(pt->ctx->stream));
    // edges of ladder l are its positions 0..n_l-2, packed ladder after ladder
    int k = 0;
    for (int l = 0; l < pt->nladders; ++l)
        for (int p = 0; p + 1 < pt->ladder_n[l]; ++p, ++k) {
            if (steps) steps[k] = s[pt->ladder_gpos0[l] + p];
            if (accepted) accepted[k] = a[pt->ladder_gpos0[l] + p];
        }
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_observables(mcx_pt* pt, int64_t* pair_sum, int64_t* spin_sum) {
    if (!pt) return fail(MCX_ERR_INVALID_ARG, "pt is NULL");
    std::vector<long long> st((size_t)pt->nrep * 2);
    MCX_CUDA(cudaMemcpyAsync(st.data(), pt->d_state, st.size() * 8, cudaMemcpyDeviceToHost, pt->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(pt->ctx->stream));
    for (int r = 0; r < pt->nrep; ++r) {
        if (pair_sum) pair_sum[r] = st[2 * r];
        if (spin_sum) spin_sum[r] = st[2 * r + 1];
    }
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_replica_accepted(mcx_pt* pt, uint64_t* accepted) {
    if (!pt || !accepted) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    MCX_CUDA(cudaMemcpyAsync(accepted, pt->d_acc, pt->nrep * 8, cudaMemcpyDeviceToHost, pt->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(pt->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_set_indices(mcx_pt* pt, const int32_t* positions, int32_t stage) {
    if (!pt || !positions) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (stage != 0 && stage != 1) return fail(MCX_ERR_INVALID_ARG, "stage must be 0 or 1");
    // every ladder must hold a permutation of its positions
    std::vector<int> seen(pt->npos, 0);
    for (int r = 0; r < pt->nrep; ++r) {
        const int l = pt->rep_ladder[r];
        const int p = positions[r];
        if (p < 0 || p >= pt->ladder_n[l] || seen[pt->ladder_gpos0[l] + p]++)
            return fail(MCX_ERR_INVALID_ARG, "positions are not a permutation within each ladder");
    }
    MCX_CUDA(cudaMemcpyAsync(pt->d_pos, positions, pt->nrep * sizeof(int32_t), cudaMemcpyHostToDevice, pt->ctx->stream));
    MCX_CUDA(cudaMemcpyAsync(pt->d_stage, &stage, sizeof(int32_t), cudaMemcpyHostToDevice, pt->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(pt->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_set_exchange_counters(mcx_pt* pt, const uint64_t* steps, const uint64_t* accepted) {
    if (!pt || !steps || !accepted) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    std::vector<unsigned long long> s(pt->npos, 0), a(pt->npos, 0);
    int k = 0;
    for (int l = 0; l < pt->nladders; ++l)
        for (int p = 0; p + 1 < pt->ladder_n[l]; ++p, ++k) {
            if (accepted[k] > steps[k]) return fail(MCX_ERR_INVALID_ARG, "accepted exceeds steps on edge %d", k);
            s[pt->ladder_gpos0[l] + p] = steps[k];
            a[pt->ladder_gpos0[l] + p] = accepted[k];
        }
    MCX_CUDA(cudaMemcpyAsync(pt->d_ex_steps, s.data(), pt->npos * 8, cudaMemcpyHostToDevice, pt->ctx->stream));
    MCX_CUDA(cudaMemcpyAsync(pt->d_ex_acc, a.data(), pt->npos * 8, cudaMemcpyHostToDevice, pt->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(pt->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_set_wait_limit(mcx_pt* pt, int64_t polls) {
    if (!pt || polls < 1) return fail(MCX_ERR_INVALID_ARG, "bad argument");
    pt->spin_limit = polls;
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_set_schedule(mcx_pt* pt, int32_t blocks_per_sm, int32_t vcap, int32_t weights) {
    if (!pt) return fail(MCX_ERR_INVALID_ARG, "pt is NULL");
    if (blocks_per_sm == 0) blocks_per_sm = pt->bps_max;
    if (blocks_per_sm < 1 || blocks_per_sm > pt->bps_max)
        return fail(MCX_ERR_INVALID_ARG, "blocks_per_sm must be in 1..%d", pt->bps_max);
    if (vcap != 16 && vcap != 8 && vcap != 4) return fail(MCX_ERR_INVALID_ARG, "vcap must be 16, 8 or 4");
    if (weights < 0 || weights > 2) return fail(MCX_ERR_INVALID_ARG, "weights must be 0, 1 or 2");
    if (pt->ctx->num_sms * blocks_per_sm * 8 < pt->nrep)
        return fail(MCX_ERR_INVALID_ARG, "%d replicas need at least as many resident warps", pt->nrep);
    return pt_apply_schedule(pt, blocks_per_sm, vcap, weights);
}

MCX_API mcx_status mcx_pt_get_schedule(const mcx_pt* pt, int32_t* blocks_per_sm, int32_t* vcap, int32_t* weights,
                                       int32_t* max_blocks_per_sm) {
    if (!pt) return fail(MCX_ERR_INVALID_ARG, "pt is NULL");
    if (blocks_per_sm) *blocks_per_sm = pt->sched_bps;
    if (vcap) *vcap = pt->sched_vcap;
    if (weights) *weights = pt->sched_weights;
    if (max_blocks_per_sm) *max_blocks_per_sm = pt->bps_max;
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_autotune(mcx_pt* pt, mcx_algorithm alg, int32_t exchange_every, int32_t sweeps,
                                   int32_t* blocks_per_sm, int32_t* vcap, int32_t* weights, double* ns_per_attempt) {
    if (!pt) return fail(MCX_ERR_INVALID_ARG, "pt is NULL");
    if (alg != MCX_METROPOLIS && alg != MCX_GLAUBER && alg != MCX_HEATBATH)
        return fail(MCX_ERR_INVALID_ARG, "unknown algorithm");
    if (exchange_every < 1 || sweeps < 1) return fail(MCX_ERR_INVALID_ARG, "exchange_every and sweeps must be >= 1");
    mcx_ctx* ctx = pt->ctx;
    cudaStream_t st = ctx->stream;
    // snapshot of everything a run changes
    const size_t sbytes = pt->arena_bytes + (size_t)pt->nrep * (2 * 8 + 4 + 8) + (size_t)pt->npos * 16 + 4;
    void* snap = nullptr;
    MCX_CHECK(dev_alloc(ctx, &snap, sbytes));
    char* sp = (char*)snap;
    struct Piece { void* dev; size_t n; };
    const Piece pieces[] = {{pt->d_arena, pt->arena_bytes}, {pt->d_state, (size_t)pt->nrep * 16},
                            {pt->d_pos, (size_t)pt->nrep * 4}, {pt->d_acc, (size_t)pt->nrep * 8},
                            {pt->d_ex_steps, (size_t)pt->npos * 8}, {pt->d_ex_acc, (size_t)pt->npos * 8},
                            {pt->d_stage, 4}};
    size_t o = 0;
    for (const Piece& q : pieces) {
        MCX_CUDA(cudaMemcpyAsync(sp + o, q.dev, q.n, cudaMemcpyDeviceToDevice, st));
        o += q.n;
    }
    const int rec = pt->record;
    const int64_t slen = pt->series_len;
    const int sbp = pt->series_by_pos;
    pt->record = 0;
    const int b0 = pt->sched_bps, v0 = pt->sched_vcap, w0 = pt->sched_weights;
    double best = 1e300;
    int bb = b0, bv = v0, bw = w0;
    mcx_status stt = MCX_OK;
    for (int b = 1; b <= pt->bps_max && stt == MCX_OK; ++b) {
        if (ctx->num_sms * b * 8 < pt->nrep) continue;
        for (int v : {16, 8})
            for (int w = 0; w < 3 && stt == MCX_OK; ++w) {
                stt = pt_apply_schedule(pt, b, v, w);
                mcx_rng r{0x5eedull, 0, 0, 0};
                if (stt == MCX_OK) stt = mcx_pt_run(pt, alg, &r, 2, exchange_every, MCX_PT_PERSISTENT, nullptr);
                double tmin = 1e300;
                for (int rep = 0; rep < 2 && stt == MCX_OK; ++rep) {
                    const auto t0 = std::chrono::steady_clock::now();
                    stt = mcx_pt_run(pt, alg, &r, sweeps, exchange_every, MCX_PT_PERSISTENT, nullptr);
                    tmin = std::min(tmin, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
                }
                if (stt == MCX_OK && tmin < best) {
                    best = tmin;
                    bb = b;
                    bv = v;
                    bw = w;
                }
            }
    }
    if (stt == MCX_OK) stt = pt_apply_schedule(pt, bb, bv, bw);
    else pt_apply_schedule(pt, b0, v0, w0);
    o = 0;
    for (const Piece& q : pieces) {
        cudaMemcpyAsync(q.dev, sp + o, q.n, cudaMemcpyDeviceToDevice, st);
        o += q.n;
    }
    cudaStreamSynchronize(st);
    dev_free(ctx, snap, sbytes);
    pt->record = rec;
    pt->series_len = slen;
    pt->series_by_pos = sbp;
    MCX_CHECK(stt);
    if (blocks_per_sm) *blocks_per_sm = bb;
    if (vcap) *vcap = bv;
    if (weights) *weights = bw;
    if (ns_per_attempt) *ns_per_attempt = best * 1e9 / ((double)pt->sites * sweeps);
    return MCX_OK;
}

MCX_API mcx_status mcx_wait_flag_test(mcx_ctx* ctx, int64_t polls) {
    if (!ctx || polls < 1) return fail(MCX_ERR_INVALID_ARG, "bad argument");
    void* p = nullptr;
    MCX_CHECK(dev_alloc(ctx, &p, 2 * sizeof(unsigned int)));
    unsigned int* d = (unsigned int*)p;
    unsigned int res = 2;
    cudaError_t e = cudaMemsetAsync(d, 0, 2 * sizeof(unsigned int), ctx->stream);
    if (e == cudaSuccess) {
        k_wait_flag<<<1, 1, 0, ctx->stream>>>(d, polls, d + 1);
        count_launch(ctx);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&res, d + 1, sizeof(res), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, p, 2 * sizeof(unsigned int));
    if (e != cudaSuccess) return cuda_fail(e, "wait-flag test");
    return res == 1 ? fail(MCX_ERR_TIMEOUT, "flag wait exceeded %lld polls", (long long)polls) : MCX_OK;
}

MCX_API mcx_status mcx_pt_set_record(mcx_pt* pt, int32_t record) {
    if (!pt) return fail(MCX_ERR_INVALID_ARG, "pt is NULL");
    if (record < 0 || record > 2) return fail(MCX_ERR_INVALID_ARG, "record must be 0, 1 or 2");
    pt->record = record;
    return MCX_OK;
}

MCX_API mcx_status mcx_pt_tau_int(mcx_pt* pt, int quantity, int64_t min_points, int64_t max_lag, double c,
                                  double* taus) {
    if (!pt || !taus) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (quantity != 0 && quantity != 1) return fail(MCX_ERR_INVALID_ARG, "quantity must be 0 (energy) or 1 (magnetization)");
    if (!(c > 0)) return fail(MCX_ERR_INVALID_ARG, "c must be positive");
    if (min_points < 2) return fail(MCX_ERR_INVALID_ARG, "min_points must be >= 2");
    if (pt->series_len == 0) return fail(MCX_ERR_INVALID_ARG, "the last run recorded no series");
    std::vector<TraceSrc> srcs(pt->nrep);
    for (int k = 0; k < pt->nrep; ++k) {
        TraceSrc& s = srcs[k];
        s = TraceSrc{};
        s.base = pt->d_series + 2 * (size_t)k;
        s.type = TRACE_I64;
        s.stride = 2 * (long long)pt->nrep;
        s.ncols = 2;
        if (quantity == 0) {  // -J pair - h spin
            s.coef[0] = -pt->J;
            s.coef[1] = -pt->h;
        } else {
            s.coef[1] = 1.0;
        }
        tau_window(s, pt->series_len, min_points, max_lag);
    }
    return launch_tau_int(pt->ctx, srcs, nullptr, 0, c, taus);
}

// One exchange stage of one ladder on the host, for a ladder whose replicas are swept by
// several processes (replica_exchange.jl:110-136 pair rule and acceptance, :158-178 stage
// order; :227-243 is the reference's MPI form, one replica per rank).  The uniforms are the
// ones the device exchange step draws (Philox counter (position, sweep, sweep>>32 |
// exchange purpose, ladder) under the ladder's seed), and the arithmetic is the device's
// in the same order, so every process taking this step with the same inputs reaches the
// same positions as k_pt_persistent.
MCX_API mcx_status mcx_ladder_exchange(int32_t n, const double* betas, const int64_t* pair_sum,
                                       const int64_t* spin_sum, double J, double h, int32_t* pos, int32_t* stage,
                                       uint64_t seed, int32_t ladder, uint64_t sweep, uint64_t* steps,
                                       uint64_t* accepted) {
    if (!betas || !pair_sum || !spin_sum || !pos || !stage || !steps || !accepted)
        return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (n < 2) return fail(MCX_ERR_INVALID_ARG, "a ladder needs at least 2 replicas");
    if (ladder < 0) return fail(MCX_ERR_INVALID_ARG, "ladder < 0");
    std::vector<int> rep(n, -1);
    for (int r = 0; r < n; ++r) {
        if (pos[r] < 0 || pos[r] >= n || rep[pos[r]] != -1)
            return fail(MCX_ERR_INVALID_ARG, "positions are not a permutation of 0..%d", n - 1);
        rep[pos[r]] = r;
    }
    for (int p = 0; p < n; ++p)
        if (!std::isfinite(betas[p])) return fail(MCX_ERR_INVALID_ARG, "beta %d must be finite", p);
    const int first = (*stage & 1) ? 1 : 0;
    for (int p = first; p + 1 < n; p += 2) {
        const int ri = rep[p], rj = rep[p + 1];
        const uint4 w = philox10(make_uint4((uint32_t)p, (uint32_t)sweep, ctr_word2(sweep, 0, P_EXCHANGE),
                                            (uint32_t)ladder),
                                 (uint32_t)seed, (uint32_t)(seed >> 32));
        const double lu = mcx_log(u53(w.x, w.y));
        const double bi = betas[p], bj = betas[p + 1];
        const double xi = (-(J * (double)pair_sum[ri])) - (h * (double)spin_sum[ri]);
        const double xj = (-(J * (double)pair_sum[rj])) - (h * (double)spin_sum[rj]);
        const double lr = (((-bi) * xj) - ((-bi) * xi)) + (((-bj) * xi) - ((-bj) * xj));
        steps[p] += 1;
        if ((lr > 0.0) || (lu < lr)) {
            accepted[p] += 1;
            pos[ri] = p + 1;
            pos[rj] = p;
        }
    }
    *stage = (*stage & 1) ^ 1;
    return MCX_OK;
}

}  // extern "C"

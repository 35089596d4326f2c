// mcx_sweep.cu -- checkerboard half-sweep kernels on the colour-split int8 layout.
//
// One launch updates every site of one colour.  A thread owns chunks of V consecutive
// sites of a row (V = 16: one 128-bit load/store per array row; V = 8 or 4 when the row
// is not a multiple of 16; V = 1 for rows that are not a multiple of 4), one chunk column
// over a run of consecutive rows in the grid kernels (strip_walk).  Neighbour sums are
// formed four sites at a time inside 32-bit words; each Philox4x32-10 call feeds the
// four sites of one word, which is exactly the counter mapping of the stream (site i
// takes word (i>>1)&3 of the call with counter (i>>3, ...)).
//
// Per-sweep energy / magnetisation deltas are reduced per block (warp shuffles)
// and added with one 64-bit atomic per block into the sweep's slot of the series.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "mcx_device.cuh"
#include "mcx_internal.h"
#include "mcx_sweep.cuh"
#include "mcx_cb.cuh"
#include "mcx_body.cuh"

namespace mcx {

// The kernel bodies below take the work items first, first + stride, ... of one
// half-sweep (the word bodies as a ChunkIter already decomposed into row and chunk;
// a.cur / a.oth may point to global or shared memory) and leave the thread's deltas
// (pair, spin, spin2, accepted) in v.  The grid kernels run one half-sweep per
// launch; k_lattice_small runs every sweep of a call in one block on a shared-memory copy.

template <int DIM, int V, bool HB, bool T32>
__device__ __forceinline__ void ising_cb_body(const SweepArgs& a, const unsigned long long* s_thr,
                                              const uint32_t* s_t32, ChunkIter it, long long (&v)[4]) {
    constexpr int Z = 2 * DIM;
    const SweepKey key = sweep_key(a);
    const uint32_t w2 = ctr_word2(key.sweep, a.colour, P_ACCEPT);
    int nacc = 0, isum = 0, nup = 0;
    for (; it.valid(); it.next()) {
        const int r = it.row();
        const int k0 = it.q * V;
        const RowInfo ri = row_info_yz(it.y, it.z, a.Ly, a.Lz, a.colour, DIM);
        Chunk<DIM, V> ch;
        ch.load(a.cur, a.oth, a.W, r, k0, ri);
        const uint32_t c0 = (uint32_t)(((unsigned long long)r * a.W + k0) >> 2);
        ising_chunk<DIM, V, HB, T32>(ch, c0, key, w2, s_thr, s_t32, nacc, nup, isum);
        store_row<V>(a.cur + (long long)r * a.W + k0, ch.own);
    }
    long long dP, dM;
    ising_deltas<Z>(nacc, nup, isum, dP, dM);
    v[0] += dP;
    v[1] += dM;
    v[3] += nacc;
}

// Column-strip walk of one half-sweep, shared by the Ising and Blume-Capel grid kernels.
// Thread (q, j) takes chunk q of a run of consecutive rows [j*rows/tpc, (j+1)*rows/tpc)
// (tpc = threads per chunk column; adjacent threads on adjacent chunks of a row).  Moving
// from row y to y+1 of a plane, the other colour's rows y and y+1 are the previous row's
// y and y+1 neighbours, so a row costs its own words, the other colour's row y+2 (and
// the two z rows in 3-D) and one edge byte, and the row, edge and counter indices
// advance by constants.  `body(ch, c0)` decides the chunk (c0 = global site index of its
// first site / 4) and leaves the new words in ch.own.  The stream does not depend on
// the walk, so results equal those of the grid-stride walk (ChunkIter).  On a GB300 this
// form beat the grid-stride walk by 4 % (2-D) and 10 % (3-D); loading the next row one
// row ahead made it 12 % slower, and the same walk inside the batched replica kernel's
// warp ranges 15 % slower.
template <int DIM, int V>
struct StripRows {
    static constexpr int NW = V / 4;
    uint32_t dn[NW], mid[NW], up[NW];
};

template <int DIM, int V, class Body>
__device__ __forceinline__ void strip_walk(const SweepArgs& a, long long tid, long long tpc, Body&& body) {
    constexpr int NW = V / 4;
    const int cpr = a.W / V;
    const int q = (int)(tid % cpr);
    const long long j = tid / cpr;
    long long r = j * a.rows / tpc;
    const long long rend = (j + 1) * a.rows / tpc;
    const int k0 = q * V;
    const int keL = k0 == 0 ? a.W - 1 : k0 - 1;  // in-row neighbour byte of a p = 0 row
    const int keR = k0 + V == a.W ? 0 : k0 + V;  // of a p = 1 row
    const long long W = a.W;
    int y = 0, p = 0;
    uint32_t c0 = 0;
    int8_t* cp = nullptr;        // own chunk of row r
    const int8_t* op = nullptr;  // the other colour's row r
    long long dzp = 0, dzm = 0;  // 3-D: offsets of the z + 1 and z - 1 rows from row r
    StripRows<DIM, V> R;
    bool fresh = true;
    for (; r < rend; ++r) {
        if (fresh || y == 0) {  // the first row of the run or of a plane
            const int z = (int)(r / a.Ly);
            y = (int)(r - (long long)z * a.Ly);
            p = (y + z + a.colour) & 1;
            c0 = (uint32_t)(((unsigned long long)r * W + k0) >> 2);
            cp = a.cur + r * W + k0;
            op = a.oth + r * W;
            if constexpr (DIM == 3) {
                dzp = (long long)((z + 1 == a.Lz ? 0 : z + 1) - z) * a.Ly * W;
                dzm = (long long)((z == 0 ? a.Lz - 1 : z - 1) - z) * a.Ly * W;
            }
            load_row<V>((y == 0 ? op + (long long)(a.Ly - 1) * W : op - W) + k0, R.dn);
            load_row<V>(op + k0, R.mid);
            fresh = false;
        } else {
#pragma unroll
            for (int w = 0; w < NW; ++w) {
                R.dn[w] = R.mid[w];
                R.mid[w] = R.up[w];
            }
        }
        load_row<V>((y + 1 == a.Ly ? op - (long long)y * W : op + W) + k0, R.up);
        Chunk<DIM, V> ch;
        load_row<V>(cp, ch.own);
#pragma unroll
        for (int w = 0; w < NW; ++w) {  // the neighbour order of Chunk::load
            ch.nb[0][w] = R.mid[w];
            ch.nb[1][w] = R.up[w];
            ch.nb[2][w] = R.dn[w];
        }
        if constexpr (DIM == 3) {
            load_row<V>(op + dzp + k0, ch.nb[4]);
            load_row<V>(op + dzm + k0, ch.nb[5]);
        }
        const uint32_t edge = (uint32_t)(uint8_t)op[p == 0 ? keL : keR];
        if (p == 0) {
#pragma unroll
            for (int w = 0; w < NW; ++w)
                ch.nb[3][w] = __funnelshift_l(w == 0 ? (edge << 24) : R.mid[w - 1], R.mid[w], 8);
        } else {
#pragma unroll
            for (int w = 0; w < NW; ++w)
                ch.nb[3][w] = __funnelshift_r(R.mid[w], w == NW - 1 ? edge : R.mid[w + 1], 8);
        }
        body(ch, c0);
        store_row<V>(cp, ch.own);
        cp += W;
        op += W;
        c0 += (uint32_t)(W >> 2);
        p ^= 1;
        if (++y == a.Ly) y = 0;
    }
}

// threads per chunk column of a launch; 0 when a row has more chunks than the grid threads
__device__ __forceinline__ long long strip_tpc(const SweepArgs& a, int V) {
    return (long long)gridDim.x * blockDim.x / (a.W / V);
}

template <int DIM, int V, bool HB, bool T32>
__global__ void __launch_bounds__(256, 2) k_ising_strip(const SweepArgs a) {
    constexpr int Z = 2 * DIM;
    constexpr int NT = 2 * (Z + 1);
    __shared__ unsigned long long s_thr[NT];
    __shared__ uint32_t s_t32[NT];
    ising_tables<DIM, HB, T32>(a, s_thr, s_t32);
    __syncthreads();
    pdl_trigger();
    pdl_wait();  // the previous half-sweep's colour array is complete
    long long v[4] = {0, 0, 0, 0};
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long tpc = strip_tpc(a, V);
    if (tpc == 0) {  // the grid-stride walk
        const ChunkIter it(tid, (long long)gridDim.x * blockDim.x, a.W / V, a.Ly, a.Lz);
        ising_cb_body<DIM, V, HB, T32>(a, s_thr, s_t32, it, v);
    } else if (tid < tpc * (a.W / V)) {
        const SweepKey key = sweep_key(a);
        const uint32_t w2 = ctr_word2(key.sweep, a.colour, P_ACCEPT);
        int nacc = 0, isum = 0, nup = 0;
        strip_walk<DIM, V>(a, tid, tpc, [&](Chunk<DIM, V>& ch, uint32_t c0) {
            ising_chunk<DIM, V, HB, T32>(ch, c0, key, w2, s_thr, s_t32, nacc, nup, isum);
        });
        long long dP, dM;
        ising_deltas<Z>(nacc, nup, isum, dP, dM);
        v[0] += dP;
        v[1] += dM;
        v[3] += nacc;
    }
    long long w[3] = {v[0], v[1], v[3]};
    const unsigned long long sh = series_shift(a);
    unsigned long long* const dst[3] = {a.dst[0] + sh, a.dst[1] + sh, a.acc};
    block_add_atomic<3>(w, dst);
}

// One site per thread, for rows whose length is not a multiple of 4.
template <int DIM, bool HB>
__device__ __forceinline__ void ising_site_body(const SweepArgs& a, const unsigned long long* s_thr, long long first,
                                                long long stride, long long (&v)[4]) {
    constexpr int Z = 2 * DIM;
    const SweepKey key = sweep_key(a);
    const unsigned long long sweep = key.sweep;
    const long long n = (long long)a.W * a.rows;
    const uint32_t w2 = ctr_word2(sweep, a.colour, P_ACCEPT);
    int nacc = 0, asum = 0, nup = 0;
    for (long long j = first; j < n; j += stride) {
        const int r = (int)(j / a.W), k = (int)(j - (long long)r * a.W);
        const RowInfo ri = row_info(r, a.Ly, a.Lz, a.colour, DIM);
        const int s = a.cur[j];
        const int ks = ri.p == 0 ? (k == 0 ? a.W - 1 : k - 1) : (k == a.W - 1 ? 0 : k + 1);
        int S = a.oth[j] + a.oth[(long long)r * a.W + ks] + a.oth[ri.ryp * a.W + k] + a.oth[ri.rym * a.W + k];
        if (DIM == 3) S += a.oth[ri.rzp * a.W + k] + a.oth[ri.rzm * a.W + k];
        const int up = s > 0;
        const int al = (s * S + Z) / 2;
        const uint4 rnd = philox10(make_uint4((uint32_t)(j >> 2), (uint32_t)sweep, w2, key.stream), key.k0, key.k1);
        uint32_t u = pick4(rnd, (int)(j & 3));
        if (HB && up) u = ~u;
        if ((unsigned long long)u < s_thr[al + (Z + 1) * up]) {
            a.cur[j] = (int8_t)(-s);
            ++nacc;
            asum += al;
            nup += up;
        }
    }
    v[0] += 2ll * Z * nacc - 4ll * asum;
    v[1] += 2ll * nacc - 4ll * nup;
    v[3] += nacc;
}

template <int DIM, bool HB>
__global__ void __launch_bounds__(256) k_ising_cb_site(const SweepArgs a) {
    constexpr int NT = 2 * (2 * DIM + 1);
    __shared__ unsigned long long s_thr[NT];
    for (int t = threadIdx.x; t < NT; t += blockDim.x) s_thr[t] = a.thr[t];
    __syncthreads();
    pdl_trigger();
    pdl_wait();
    long long v[4] = {0, 0, 0, 0};
    ising_site_body<DIM, HB>(a, s_thr, blockIdx.x * (long long)blockDim.x + threadIdx.x,
                             (long long)gridDim.x * blockDim.x, v);
    long long w[3] = {v[0], v[1], v[3]};
    const unsigned long long sh = series_shift(a);
    unsigned long long* const dst[3] = {a.dst[0] + sh, a.dst[1] + sh, a.acc};
    block_add_atomic<3>(w, dst);
}

// ------------------------------------------------------------ Blume-Capel --
template <int DIM, int V, bool HB>
__device__ __forceinline__ void bc_cb_body(const SweepArgs& a, const unsigned long long* s_thr, ChunkIter it,
                                           long long (&v)[4]) {
    const SweepKey key = sweep_key(a);
    const uint32_t w2a = ctr_word2(key.sweep, a.colour, P_ACCEPT);
    const uint32_t w2p = ctr_word2(key.sweep, a.colour, a.planes ? P_PLANES : P_PROPOSE);
    int nacc = 0, dP = 0, dM = 0, dQ = 0;
    for (; it.valid(); it.next()) {
        const int r = it.row();
        const int k0 = it.q * V;
        const RowInfo ri = row_info_yz(it.y, it.z, a.Ly, a.Lz, a.colour, DIM);
        Chunk<DIM, V> ch;
        ch.load(a.cur, a.oth, a.W, r, k0, ri);
        const uint32_t c0 = (uint32_t)(((unsigned long long)r * a.W + k0) >> 2);
        bc_chunk<DIM, V, HB>(ch, c0, key, w2a, w2p, a.planes != 0, s_thr, nacc, dP, dM, dQ);
        store_row<V>(a.cur + (long long)r * a.W + k0, ch.own);
    }
    v[0] += dP;
    v[1] += dM;
    v[2] += dQ;
    v[3] += nacc;
}

// PL: the proposal bits from bit planes (the lattice's form, compiled in on this path).
template <int DIM, int V, bool HB, bool PL = false>
__global__ void __launch_bounds__(256, 2) k_bc_strip(const SweepArgs a) {
    constexpr int NT = bc_table_size<DIM, HB>();
    __shared__ __align__(16) unsigned long long s_thr[NT];
    for (int t = threadIdx.x; t < NT; t += blockDim.x) s_thr[t] = a.thr[t];
    __syncthreads();
    pdl_trigger();
    pdl_wait();
    long long v[4] = {0, 0, 0, 0};
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long tpc = strip_tpc(a, V);
    if (tpc == 0) {  // the grid-stride walk
        const ChunkIter it(tid, (long long)gridDim.x * blockDim.x, a.W / V, a.Ly, a.Lz);
        bc_cb_body<DIM, V, HB>(a, s_thr, it, v);
    } else if (tid < tpc * (a.W / V)) {
        const SweepKey key = sweep_key(a);
        const uint32_t w2a = ctr_word2(key.sweep, a.colour, P_ACCEPT);
        const uint32_t w2p = ctr_word2(key.sweep, a.colour, PL ? P_PLANES : P_PROPOSE);
        int nacc = 0, dP = 0, dM = 0, dQ = 0;
        strip_walk<DIM, V>(a, tid, tpc, [&](Chunk<DIM, V>& ch, uint32_t c0) {
            bc_chunk<DIM, V, HB, PL ? 1 : 0>(ch, c0, key, w2a, w2p, PL, s_thr, nacc, dP, dM, dQ);
        });
        v[0] += dP;
        v[1] += dM;
        v[2] += dQ;
        v[3] += nacc;
    }
    const unsigned long long sh = series_shift(a);
    unsigned long long* const dst[4] = {a.dst[0] + sh, a.dst[1] + sh, a.dst[2] + sh, a.acc};
    block_add_atomic<4>(v, dst);
}

template <int DIM, bool HB>
__device__ __forceinline__ void bc_site_body(const SweepArgs& a, const unsigned long long* s_thr, long long first,
                                             long long stride, long long (&v)[4]) {
    constexpr int Z = 2 * DIM;
    constexpr int NC = 2 * Z + 1;
    const SweepKey key = sweep_key(a);
    const unsigned long long sweep = key.sweep;
    const long long n = (long long)a.W * a.rows;
    const uint32_t w2a = ctr_word2(sweep, a.colour, P_ACCEPT);
    const uint32_t w2p = ctr_word2(sweep, a.colour, a.planes ? P_PLANES : P_PROPOSE);
    int nacc = 0, dP = 0, dM = 0, dQ = 0;
    for (long long j = first; j < n; j += stride) {
        const int r = (int)(j / a.W), k = (int)(j - (long long)r * a.W);
        const RowInfo ri = row_info(r, a.Ly, a.Lz, a.colour, DIM);
        const int so = a.cur[j];
        const int ks = ri.p == 0 ? (k == 0 ? a.W - 1 : k - 1) : (k == a.W - 1 ? 0 : k + 1);
        int c = a.oth[j] + a.oth[(long long)r * a.W + ks] + a.oth[ri.ryp * a.W + k] + a.oth[ri.rym * a.W + k];
        if (DIM == 3) c += a.oth[ri.rzp * a.W + k] + a.oth[ri.rzm * a.W + k];
        const int S = c + Z;
        const uint32_t u = pick4(philox10(make_uint4((uint32_t)(j >> 2), (uint32_t)sweep, w2a, key.stream), key.k0, key.k1), (int)(j & 3));
        int sn;
        bool acc;
        if (HB) {
            sn = (unsigned long long)u < s_thr[2 * S] ? -1 : ((unsigned long long)u < s_thr[2 * S + 1] ? 0 : 1);
            acc = sn != so;
        } else {
            int bit;
            if (a.planes) {  // bit j & 63 of plane j >> 6: half (j >> 6) & 1 of the block at j >> 7
                const uint4 b = philox10(make_uint4((uint32_t)(j >> 7), (uint32_t)sweep, w2p, key.stream), key.k0, key.k1);
                const uint32_t half = (j >> 5) & 1 ? ((j >> 6) & 1 ? b.w : b.y) : ((j >> 6) & 1 ? b.z : b.x);
                bit = (int)((half >> (j & 31)) & 1u);
            } else {
                const uint32_t pw = pick4(philox10(make_uint4((uint32_t)(j >> 2), (uint32_t)sweep, w2p, key.stream), key.k0, key.k1), (int)(j & 3));
                bit = (int)(pw >> 31);
            }
            acc = (unsigned long long)u < s_thr[(so + 1) * 2 * NC + bit * NC + S];
            sn = bc_propose(so, bit);
        }
        if (acc) {
            const int ds = sn - so;
            a.cur[j] = (int8_t)sn;
            ++nacc;
            dP += ds * c;
            dM += ds;
            dQ += sn * sn - so * so;
        }
    }
    v[0] += dP;
    v[1] += dM;
    v[2] += dQ;
    v[3] += nacc;
}

template <int DIM, bool HB>
__global__ void __launch_bounds__(256) k_bc_cb_site(const SweepArgs a) {
    constexpr int NT = bc_table_size<DIM, HB>();
    __shared__ unsigned long long s_thr[NT];
    for (int t = threadIdx.x; t < NT; t += blockDim.x) s_thr[t] = a.thr[t];
    __syncthreads();
    pdl_trigger();
    pdl_wait();
    long long v[4] = {0, 0, 0, 0};
    bc_site_body<DIM, HB>(a, s_thr, blockIdx.x * (long long)blockDim.x + threadIdx.x,
                          (long long)gridDim.x * blockDim.x, v);
    const unsigned long long sh = series_shift(a);
    unsigned long long* const dst[4] = {a.dst[0] + sh, a.dst[1] + sh, a.dst[2] + sh, a.acc};
    block_add_atomic<4>(v, dst);
}

// ------------------------------------------------------ small lattices --
// Every sweep of one call in one block of 512 threads: both colour arrays are copied
// to shared memory, each half-sweep runs the body above on them (the neighbours of a
// colour are the other colour's array, finished by the previous half-sweep; a
// __syncthreads separates them), and each sweep's deltas go to its series slot with one
// atomic per value.  One launch per call: no per-half-sweep launch and no graph capture.
// One SM issues about 2.4e11 thread-instructions per second and a site costs about 30, so
// this pays up to about 16K sites; the rows are taken four sites at a time (the shortest
// dependent chain per thread: latency, not issue, bounds a half-sweep this small).
// KIND: 0 Ising words, 1 Ising per site, 2 Blume-Capel words, 3 Blume-Capel per site.
template <int KIND, int DIM, int V, bool HB, bool T32>
__device__ __forceinline__ void lattice_small_run(const SweepArgs& a0, int8_t* g0, int8_t* g1, long long half,
                                                  long long nsweeps, long long* series) {
    extern __shared__ __align__(16) int8_t s_lat[];
    __shared__ __align__(16) unsigned long long s_thr[kMaxTable];
    __shared__ uint32_t s_t32[kMaxTable];
    const long long off1 = (half + 15) & ~15ll;
    int8_t* s0 = s_lat;
    int8_t* s1 = s_lat + off1;
    if (half % 16 == 0) {
        for (long long i = threadIdx.x; i < half / 16; i += blockDim.x) {
            reinterpret_cast<uint4*>(s0)[i] = reinterpret_cast<const uint4*>(g0)[i];
            reinterpret_cast<uint4*>(s1)[i] = reinterpret_cast<const uint4*>(g1)[i];
        }
    } else {
        for (long long i = threadIdx.x; i < half; i += blockDim.x) {
            s0[i] = g0[i];
            s1[i] = g1[i];
        }
    }
    if constexpr (KIND == 0) {
        ising_tables<DIM, HB, T32>(a0, s_thr, s_t32);
    } else {
        for (int t = threadIdx.x; t < kMaxTable; t += blockDim.x) s_thr[t] = a0.thr[t];
    }
    __syncthreads();
    SweepArgs a;  // the fields the bodies read (the table is in shared memory)
    a.W = a0.W;
    a.Ly = a0.Ly;
    a.Lz = a0.Lz;
    a.rows = a0.rows;
    a.k0 = a0.k0;
    a.k1 = a0.k1;
    a.stream = a0.stream;
    a.planes = a0.planes;
    a.sweep_base = nullptr;
    a.acc = a0.acc;
    const unsigned long long sweep0 = a0.sweep;
    // this thread's chunks are the same in every half-sweep: decompose them once
    const ChunkIter it0(threadIdx.x, blockDim.x, a0.W / V, a0.Ly, a0.Lz);
    for (long long t = 0; t < nsweeps; ++t) {
        long long v[4] = {0, 0, 0, 0};
        for (int c = 0; c < 2; ++c) {
            a.colour = c;
            a.cur = c ? s1 : s0;
            a.oth = c ? s0 : s1;
            a.sweep = sweep0 + (unsigned long long)t;
            if constexpr (KIND == 0) ising_cb_body<DIM, V, HB, T32>(a, s_thr, s_t32, it0, v);
            else if constexpr (KIND == 1) ising_site_body<DIM, HB>(a, s_thr, threadIdx.x, blockDim.x, v);
            else if constexpr (KIND == 2) bc_cb_body<DIM, V, HB>(a, s_thr, it0, v);
            else bc_site_body<DIM, HB>(a, s_thr, threadIdx.x, blockDim.x, v);
            __syncthreads();
        }
        unsigned long long* const dst[4] = {(unsigned long long*)(series + 3 * t), (unsigned long long*)(series + 3 * t + 1),
                                            (unsigned long long*)(series + 3 * t + 2), a.acc};
        warp_add_atomic<4>(v, dst);  // half <= 8192: per-warp sums fit in int32
    }
    if (half % 16 == 0) {
        for (long long i = threadIdx.x; i < half / 16; i += blockDim.x) {
            reinterpret_cast<uint4*>(g0)[i] = reinterpret_cast<const uint4*>(s0)[i];
            reinterpret_cast<uint4*>(g1)[i] = reinterpret_cast<const uint4*>(s1)[i];
        }
    } else {
        for (long long i = threadIdx.x; i < half; i += blockDim.x) {
            g0[i] = s0[i];
            g1[i] = s1[i];
        }
    }
}

template <int KIND, int DIM, int V, bool HB, bool T32>
__global__ void __launch_bounds__(512, 1) k_lattice_small(SweepArgs a, int8_t* g0, int8_t* g1, long long half,
                                                          long long nsweeps, long long* series) {
    lattice_small_run<KIND, DIM, V, HB, T32>(a, g0, g1, half, nsweeps, series);
}

// Many independent small lattices (the chains of a ParallelChains with a threads backend,
// src/infrastructure/parallel_chains.jl:99-105) in one launch: block b runs every sweep of
// lattice b as k_lattice_small does, after zeroing that lattice's series slots and counter.
struct SmallBatchDesc {
    SweepArgs a;  // the lattice's geometry, key, table (its beta) and counter
    int8_t* col0;
    int8_t* col1;
    long long half;
    long long* series;
    long long* state;
};

// 256 threads and up to two lattices per SM: with more chains than SMs this hides more
// latency than one 512-thread block per SM (608 chains of 64^2: +28 %)
template <int KIND, int DIM, int V, bool HB, bool T32>
__global__ void __launch_bounds__(256, 2) k_lattice_small_batch(const SmallBatchDesc* __restrict__ descs,
                                                                long long nsweeps) {
    const SmallBatchDesc& d = descs[blockIdx.x];
    for (long long i = threadIdx.x; i < 3 * nsweeps; i += blockDim.x) d.series[i] = 0;
    if (threadIdx.x == 0) *d.a.acc = 0ull;
    __syncthreads();
    lattice_small_run<KIND, DIM, V, HB, T32>(d.a, d.col0, d.col1, d.half, nsweeps, d.series);
}

// the prefix sum of k_prefix_series for every lattice of a batch (block b: lattice b)
__global__ void k_prefix_series_batch(const SmallBatchDesc* __restrict__ descs, long long n) {
    const SmallBatchDesc& d = descs[blockIdx.x];
    const int j = threadIdx.x;
    if (j >= 3) return;
    long long acc = d.state[j];
    for (long long s = 0; s < n; ++s) {
        acc += d.series[3 * s + j];
        d.series[3 * s + j] = acc;
    }
    d.state[j] = acc;
}

// ----------------------------------------------------------- dispatching --
template <int DIM, bool T32>
static HalfSweepFn pick_ising_word(bool hb, int V) {
    if (V == 16) return hb ? k_ising_strip<DIM, 16, true, T32> : k_ising_strip<DIM, 16, false, T32>;
    if (V == 8) return hb ? k_ising_strip<DIM, 8, true, T32> : k_ising_strip<DIM, 8, false, T32>;
    return hb ? k_ising_strip<DIM, 4, true, T32> : k_ising_strip<DIM, 4, false, T32>;
}

template <int DIM>
static HalfSweepFn pick_kernel_dim(mcx_model model, mcx_algorithm alg, int V, const Table& t, bool planes) {
    const bool hb = alg == MCX_HEATBATH;
    if (model == MCX_ISING) {
        if (V == 16 || V == 8 || V == 4)
            return ising_table_fits32(t.thr, t.n, 2 * DIM, hb) ? pick_ising_word<DIM, true>(hb, V)
                                                               : pick_ising_word<DIM, false>(hb, V);
        return hb ? k_ising_cb_site<DIM, true> : k_ising_cb_site<DIM, false>;
    }
    // Metropolis / Glauber: the proposal form compiled in (plane or per-site proposal bits)
    if (V == 16) return hb ? k_bc_strip<DIM, 16, true> : planes ? k_bc_strip<DIM, 16, false, true> : k_bc_strip<DIM, 16, false>;
    if (V == 8) return hb ? k_bc_strip<DIM, 8, true> : planes ? k_bc_strip<DIM, 8, false, true> : k_bc_strip<DIM, 8, false>;
    if (V == 4) return hb ? k_bc_strip<DIM, 4, true> : planes ? k_bc_strip<DIM, 4, false, true> : k_bc_strip<DIM, 4, false>;
    return hb ? k_bc_cb_site<DIM, true> : k_bc_cb_site<DIM, false>;
}

// The half-sweep kernel of `lat` (its dimension, model and, for Blume-Capel, uniforms form).
HalfSweepFn pick_half_sweep(const mcx_lattice* lat, mcx_algorithm alg, int V, const Table& t) {
    const bool planes = lat->model == MCX_BLUME_CAPEL && lat->uniforms == MCX_UNIFORMS_PLANES;
    return lat->dim == 2 ? pick_kernel_dim<2>(lat->model, alg, V, t, planes)
                         : pick_kernel_dim<3>(lat->model, alg, V, t, planes);
}

using SmallLatticeFn = void (*)(SweepArgs, int8_t*, int8_t*, long long, long long, long long*);

// The chunk width of the one-block and cluster kernels: the widest V in {16, 8} that
// divides the row and still leaves at least 256 chunks of the sites of a colour one block
// holds, else 4.  Wider chunks share the
// per-chunk row and address work over more sites; 256 chunks keep enough warps busy on
// the one SM (64^2: V = 8 on 256 threads, 9 % faster than V = 4; 128^2: V = 16 on 512
// threads, 25 % faster; identical results, the stream does not depend on V).
int small_width(int64_t W, long long sites) {
    for (int V : {16, 8})
        if (W % V == 0 && sites / V >= 256) return V;
    return 4;
}

template <template <int, int, int, bool, bool> class K, int DIM, bool HB>
static typename K<0, DIM, 4, HB, false>::Fn pick_small_kind(int kind, bool t32, int V) {
    if (kind == 0) {
        if (V == 16) return t32 ? K<0, DIM, 16, HB, true>::fn : K<0, DIM, 16, HB, false>::fn;
        if (V == 8) return t32 ? K<0, DIM, 8, HB, true>::fn : K<0, DIM, 8, HB, false>::fn;
        return t32 ? K<0, DIM, 4, HB, true>::fn : K<0, DIM, 4, HB, false>::fn;
    }
    if (kind == 1) return K<1, DIM, 1, HB, false>::fn;
    if (kind == 2) {
        if (V == 16) return K<2, DIM, 16, HB, false>::fn;
        if (V == 8) return K<2, DIM, 8, HB, false>::fn;
        return K<2, DIM, 4, HB, false>::fn;
    }
    return K<3, DIM, 1, HB, false>::fn;
}

using SmallLatticeFn = void (*)(SweepArgs, int8_t*, int8_t*, long long, long long, long long*);
using SmallBatchFn = void (*)(const SmallBatchDesc*, long long);

template <int KIND, int DIM, int V, bool HB, bool T32>
struct SingleK {
    using Fn = SmallLatticeFn;
    static constexpr Fn fn = k_lattice_small<KIND, DIM, V, HB, T32>;
};
template <int KIND, int DIM, int V, bool HB, bool T32>
struct BatchK {
    using Fn = SmallBatchFn;
    static constexpr Fn fn = k_lattice_small_batch<KIND, DIM, V, HB, T32>;
};

template <template <int, int, int, bool, bool> class K>
static typename K<0, 2, 4, false, false>::Fn pick_small_fn(int dim, bool hb, int kind, bool t32, int V) {
    if (dim == 2) return hb ? pick_small_kind<K, 2, true>(kind, t32, V) : pick_small_kind<K, 2, false>(kind, t32, V);
    return hb ? pick_small_kind<K, 3, true>(kind, t32, V) : pick_small_kind<K, 3, false>(kind, t32, V);
}

static int small_kind(mcx_model model, bool words) { return model == MCX_ISING ? (words ? 0 : 1) : (words ? 2 : 3); }

int vec_width(int64_t W) { return W % 16 == 0 ? 16 : (W % 8 == 0 ? 8 : (W % 4 == 0 ? 4 : 1)); }

int lattice_width(const mcx_lattice* lat) {
    const int V = lat->tuned_V;
    return (V > 0 && lat->W % V == 0) ? V : vec_width(lat->W);
}

// Grid = min(work, SMs x resident blocks per SM): one wave of a grid-stride kernel.
int occupancy_grid(const mcx_ctx* ctx, const void* fn, long long work, int block, size_t smem) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, int> cache;
    int bps = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto key = std::make_pair(fn, block);
        auto it = cache.find(key);
        if (it != cache.end()) {
            bps = it->second;
        } else {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, block, smem) != cudaSuccess) bps = 1;
            cache[key] = bps;
        }
    }
    long long g = (work + block - 1) / block;
    const long long cap = (long long)ctx->num_sms * (bps > 0 ? bps : 1);
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

int half_sweep_grid(const mcx_ctx* ctx, HalfSweepFn fn, int64_t W, int64_t rows, int V) {
    return occupancy_grid(ctx, (const void*)fn, (long long)(W / V) * rows, 256, 0);
}

mcx_status build_table(const mcx_lattice* lat, mcx_algorithm alg, double beta, Table* t) {
    if (lat->model == MCX_ISING) return build_ising_table(lat->dim, alg, beta, lat->J, lat->h, t);
    return build_bc_table(lat->dim, alg, beta, lat->J, lat->D, lat->h, t);
}

void fill_sweep_args(SweepArgs* a, const mcx_lattice* lat, const Table& t, const mcx_rng* rng) {
    a->sweep_base = nullptr;
    a->W = (int)lat->W;
    a->Ly = (int)lat->L[1];
    a->Lz = (int)lat->L[2];
    a->rows = (int)lat->rows;
    a->k0 = (uint32_t)rng->seed;
    a->k1 = (uint32_t)(rng->seed >> 32);
    a->stream = rng->stream;
    for (int i = 0; i < t.n; ++i) a->thr[i] = t.thr[i];
    a->planes = lat->model == MCX_BLUME_CAPEL && lat->uniforms == MCX_UNIFORMS_PLANES;
}

mcx_status msc_sweep(mcx_lattice* lat, mcx_algorithm alg, const Table& t, const mcx_rng* rng,
                     int64_t nsweeps);  // mcx_msc.cu
bool msc_transient_ok(mcx_lattice* lat, mcx_algorithm alg, const Table& t);  // mcx_msc.cu
mcx_status msc_pack(mcx_lattice* lat);                                       // mcx_msc.cu
mcx_status msc_unpack(mcx_lattice* lat);                                     // mcx_msc.cu
mcx_status msc_planes_copy(mcx_lattice* lat);                                // mcx_msc.cu

__global__ void k_set_key(unsigned long long* p, unsigned long long sweep, unsigned long long seed,
                          unsigned long long stream) {
    p[0] = sweep;
    p[1] = seed;
    p[2] = stream;
    p[3] = 0;
}

// last node of a captured chunk: the next replay continues where this one stopped
__global__ void k_advance_key(unsigned long long* p, unsigned long long n) {
    p[0] += n;
    p[3] += n;
}

// kGraphChunk sweeps (2 * kGraphChunk half-sweeps, then k_advance_key) captured once
// into a CUDA graph on a private stream.  The kernels read the first sweep, the Philox key
// and the series offset from lat->d_sweep_base, so the instantiated graph serves every
// call with the same algorithm and beta, whatever its length or random stream: a call
// replays it back to back and launches the remainder directly.  (Capturing the whole
// sequence of a call cost about 10 us per sweep for every new length.)
// One half-sweep launch; `dependent`: programmatic dependency on the launch before it in
// the stream (the kernels read the lattice only after pdl_wait).
static cudaError_t launch_half(HalfSweepFn fn, int grid, cudaStream_t st, const SweepArgs& a, bool dependent) {
    cudaLaunchAttribute pdl[1];
    pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cfg.attrs = pdl;
    cfg.numAttrs = dependent ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, fn, a);
}

static mcx_status sweep_graph(mcx_lattice* lat, mcx_algorithm alg, double beta, const Table& t, int V,
                              cudaGraphExec_t* out) {
    for (auto& g : lat->graphs)
        if (g.alg == (int)alg && g.uniforms == lat->uniforms && g.beta == beta && g.V == V && g.series == lat->d_series) {
            *out = g.exec;
            return MCX_OK;
        }
    mcx_ctx* ctx = lat->ctx;
    if (!ctx->capture_stream) MCX_CUDA(cudaStreamCreateWithFlags(&ctx->capture_stream, cudaStreamNonBlocking));
    cudaStream_t cs = ctx->capture_stream;
    SweepArgs a;
    mcx_rng r0{0, 0, 0, 0};
    fill_sweep_args(&a, lat, t, &r0);
    a.sweep_base = lat->d_sweep_base;
    a.acc = lat->d_acc;
    const HalfSweepFn fn = pick_half_sweep(lat, alg, V, t);
    const int grid = half_sweep_grid(ctx, fn, lat->W, lat->rows, V);
    // Each half-sweep node after the first depends programmatically on the one before: its
    // blocks may be scheduled, and build their tables, while the previous half-sweep drains;
    // they read the lattice only after pdl_wait.  The key-advancing node depends fully.
    MCX_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    for (int64_t s = 0; s < kGraphChunk; ++s) {
        a.sweep = (uint64_t)s;
        for (int c = 0; c < 2; ++c) {
            a.colour = c;
            a.cur = lat->d_col[c];
            a.oth = lat->d_col[1 - c];
            for (int j = 0; j < 3; ++j) a.dst[j] = (unsigned long long*)(lat->d_series + 3 * s + j);
            if (le == cudaSuccess) le = launch_half(fn, grid, cs, a, s > 0 || c > 0);
        }
    }
    k_advance_key<<<1, 1, 0, cs>>>(lat->d_sweep_base, (unsigned long long)kGraphChunk);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &graph);
    if (e == cudaSuccess) e = le;
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "sweep graph capture");
    if (lat->graphs.size() >= 4) {
        cudaGraphExecDestroy(lat->graphs.front().exec);
        lat->graphs.erase(lat->graphs.begin());
    }
    lat->graphs.push_back({(int)alg, lat->uniforms, beta, kGraphChunk, V, lat->d_series, exec});
    *out = exec;
    return MCX_OK;
}

}  // namespace mcx

using namespace mcx;

extern "C" MCX_API mcx_status mcx_sweep(mcx_lattice* lat, mcx_algorithm alg, double beta, mcx_rng* rng,
                                        int64_t nsweeps, int64_t* obs, mcx_counters* counters) {
    if (!lat || !rng) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (nsweeps < 0) return fail(MCX_ERR_INVALID_ARG, "nsweeps < 0");
    if (!std::isfinite(beta)) return fail(MCX_ERR_INVALID_ARG, "beta must be finite");
    if (alg != MCX_METROPOLIS && alg != MCX_GLAUBER && alg != MCX_HEATBATH)
        return fail(MCX_ERR_INVALID_ARG, "unknown algorithm %d", (int)alg);
    if (rng->counter + (uint64_t)nsweeps >= (1ull << 48))
        return fail(MCX_ERR_INVALID_ARG, "sweep counter beyond 2^48");
    mcx_ctx* ctx = lat->ctx;
    Table t;
    MCX_CHECK(build_table(lat, alg, beta, &t));
    MCX_CHECK(ensure_series(lat, nsweeps > 0 ? nsweeps : 1));
    // medium int8 lattices run every sweep of the call in one thread-block cluster, small
    // ones (and those the cluster form does not take, up to kSmallLattice sites) in one
    // block; larger ones replay a captured chunk of kGraphChunk sweeps as often as it fits
    // and launch the rest directly
    // With per-site uniforms MSC64 lattices sweep the packed words only under k_msc_metro's
    // rank or class form (Metropolis or Glauber without a field); other rules run on their
    // int8 arrays (unpacked before, packed after the call), which is faster than a per-site
    // table lookup on the words.
    // With bit-plane uniforms every Ising call runs on the words: an int8 lattice's on its
    // transient copy, whatever the call's length (the int8 kernels draw per-site words).
    const bool pl_rule = msc_planes_ok(lat, alg, t);  // every Ising rule under bit-plane uniforms
    const bool msc_words = lat->layout == MCX_LAYOUT_MSC64 && (pl_rule || msc_rank_ok(lat, alg, t));
    const bool via_int8 = lat->layout == MCX_LAYOUT_MSC64 && !msc_words;
    const bool int8 = lat->layout == MCX_LAYOUT_INT8 || via_int8;
    const bool planes = lat->layout == MCX_LAYOUT_INT8 && pl_rule && nsweeps > 0;
    if (planes) MCX_CHECK(msc_planes_copy(lat));
    if (via_int8) MCX_CHECK(msc_unpack(lat));
    MCX_CUDA(cudaMemsetAsync(lat->d_series, 0, (size_t)nsweeps * 3 * sizeof(int64_t), ctx->stream));
    MCX_CUDA(cudaMemsetAsync(lat->d_acc, 0, sizeof(unsigned long long), ctx->stream));
    // large int8 Ising lattices under Metropolis or Glauber without a field run calls of
    // kMscMinSweeps sweeps or more on a transient 64-sites-per-word copy (k_msc_metro: 1.8x
    // and 1.46x the int8 words; packing and unpacking cost about two sweeps' worth of
    // one-pass copies)
    const bool transient = planes || (int8 && lat->N > kClusterLattice && nsweeps >= kMscMinSweeps &&
                                      msc_transient_ok(lat, alg, t));
    bool clustered = false;
    if (!transient && int8 && lat->N > kClusterMin) MCX_CHECK(cluster_sweep(lat, alg, t, rng, nsweeps, &clustered));
    const bool small = !transient && !clustered && int8 && lat->N <= kSmallLattice && nsweeps >= 1;
    const bool graph = !transient && !small && !clustered && int8 && nsweeps >= kGraphChunk;
    if (clustered) {
        // launched by cluster_sweep
    } else if (transient) {
        MCX_CHECK(msc_pack(lat));
        MCX_CHECK(msc_sweep(lat, alg, t, rng, nsweeps));
        MCX_CHECK(msc_unpack(lat));
    } else if (msc_words) {
        MCX_CHECK(msc_sweep(lat, alg, t, rng, nsweeps));
    } else if (small) {
        SweepArgs a;
        fill_sweep_args(&a, lat, t, rng);
        a.acc = lat->d_acc;
        a.sweep = rng->counter;
        const long long half = lat->N / 2;
        const bool hb = alg == MCX_HEATBATH;
        const int kind = small_kind(lat->model, lat->W % 4 == 0);
        const bool t32 = kind == 0 && ising_table_fits32(t.thr, t.n, 2 * lat->dim, hb);
        const int V = (kind == 0 || kind == 2) ? small_width(lat->W, half) : 1;
        const SmallLatticeFn fn = pick_small_fn<SingleK>(lat->dim, hb, kind, t32, V);
        // one thread per chunk up to 512 (whole warps)
        const int threads = V == 1 ? 512 : (int)std::min<long long>(512, std::max<long long>(32, (half / V + 31) & ~31ll));
        const size_t smem = (size_t)(((half + 15) & ~15ll) + half);
        if (smem > 48 * 1024)
            MCX_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        fn<<<1, threads, smem, ctx->stream>>>(a, lat->d_col[0], lat->d_col[1], half, nsweeps,
                                           reinterpret_cast<long long*>(lat->d_series));
        count_launch(ctx);
        MCX_CUDA(cudaGetLastError());
    } else if (graph) {
        const int V = lattice_width(lat);
        cudaGraphExec_t exec = nullptr;
        MCX_CHECK(sweep_graph(lat, alg, beta, t, V, &exec));
        k_set_key<<<1, 1, 0, ctx->stream>>>(lat->d_sweep_base, (unsigned long long)rng->counter,
                                            (unsigned long long)rng->seed, (unsigned long long)rng->stream);
        MCX_CUDA(cudaGetLastError());
        const int64_t q = nsweeps / kGraphChunk, rem = nsweeps - q * kGraphChunk;
        for (int64_t i = 0; i < q; ++i) MCX_CUDA(cudaGraphLaunch(exec, ctx->stream));
        count_launch(ctx, 1 + (uint64_t)q * (2 * kGraphChunk + 1));
        if (rem > 0) {  // relative to the advanced key: sweeps q*C .. of the call, slots likewise
            SweepArgs a;
            fill_sweep_args(&a, lat, t, rng);
            a.sweep_base = lat->d_sweep_base;
            a.acc = lat->d_acc;
            const HalfSweepFn fn = pick_half_sweep(lat, alg, V, t);
            const int grid = half_sweep_grid(ctx, fn, lat->W, lat->rows, V);
            for (int64_t s = 0; s < rem; ++s) {
                a.sweep = (uint64_t)s;
                for (int c = 0; c < 2; ++c) {
                    a.colour = c;
                    a.cur = lat->d_col[c];
                    a.oth = lat->d_col[1 - c];
                    for (int j = 0; j < 3; ++j) a.dst[j] = (unsigned long long*)(lat->d_series + 3 * s + j);
                    MCX_CUDA(launch_half(fn, grid, ctx->stream, a, s > 0 || c > 0));
                }
            }
            count_launch(ctx, 2 * (uint64_t)rem);
            MCX_CUDA(cudaGetLastError());
        }
    } else {
        SweepArgs a;
        fill_sweep_args(&a, lat, t, rng);
        a.acc = lat->d_acc;
        const int V = lattice_width(lat);
        const HalfSweepFn fn = pick_half_sweep(lat, alg, V, t);
        const int grid = half_sweep_grid(ctx, fn, lat->W, lat->rows, V);
        for (int64_t s = 0; s < nsweeps; ++s) {
            a.sweep = rng->counter + (uint64_t)s;
            for (int c = 0; c < 2; ++c) {
                a.colour = c;
                a.cur = lat->d_col[c];
                a.oth = lat->d_col[1 - c];
                for (int j = 0; j < 3; ++j) a.dst[j] = (unsigned long long*)(lat->d_series + 3 * s + j);
                MCX_CUDA(launch_half(fn, grid, ctx->stream, a, s > 0 || c > 0));
            }
        }
        count_launch(ctx, 2 * (uint64_t)nsweeps);
        MCX_CUDA(cudaGetLastError());
    }
    if (via_int8) MCX_CHECK(msc_pack(lat));
    MCX_CHECK(finish_series(lat, nsweeps));
    rng->counter += (uint64_t)nsweeps;
    if (obs && nsweeps > 0)
        MCX_CUDA(cudaMemcpyAsync(obs, lat->d_series, (size_t)nsweeps * 3 * sizeof(int64_t),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    if (counters) {
        unsigned long long acc = 0;
        MCX_CUDA(cudaMemcpyAsync(&acc, lat->d_acc, sizeof(acc), cudaMemcpyDeviceToHost, ctx->stream));
        MCX_CUDA(cudaStreamSynchronize(ctx->stream));
        counters->attempts += (uint64_t)lat->N * (uint64_t)nsweeps;
        counters->accepted += acc;
    } else if (obs) {
        MCX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return MCX_OK;
}

// ------------------------------------------------------------- autotuning --
// Times every admissible row width (16, 8, 4 sites per thread; 1 only when nothing
// else fits) on a scratch copy of the lattice and keeps the fastest for later
// mcx_sweep calls.  The choice never changes results: every width applies the same
// stream to the same sites.
extern "C" MCX_API mcx_status mcx_autotune(mcx_lattice* lat, mcx_algorithm alg, double beta, int32_t* chosen,
                                           double* ns_per_site) {
    if (!lat) return fail(MCX_ERR_INVALID_ARG, "lattice is NULL");
    if (!std::isfinite(beta)) return fail(MCX_ERR_INVALID_ARG, "beta must be finite");
    if (alg != MCX_METROPOLIS && alg != MCX_GLAUBER && alg != MCX_HEATBATH)
        return fail(MCX_ERR_INVALID_ARG, "unknown algorithm %d", (int)alg);
    if (lat->layout != MCX_LAYOUT_INT8) {
        if (chosen) *chosen = 64;
        if (ns_per_site) *ns_per_site = 0.0;
        return MCX_OK;
    }
    mcx_ctx* ctx = lat->ctx;
    std::vector<int> cands;
    for (int V : {16, 8, 4})
        if (lat->W % V == 0) cands.push_back(V);
    if (cands.empty()) cands.push_back(1);
    Table t;
    MCX_CHECK(build_table(lat, alg, beta, &t));
    const size_t half = (size_t)(lat->N / 2);
    void* scratch = nullptr;
    const size_t bytes = 2 * ((half + 255) / 256 * 256) + 3 * 8 + 8;
    MCX_CHECK(dev_alloc(ctx, &scratch, bytes));
    int8_t* col[2] = {(int8_t*)scratch, (int8_t*)scratch + (half + 255) / 256 * 256};
    unsigned long long* acc = (unsigned long long*)(col[1] + (half + 255) / 256 * 256);
    unsigned long long* dst = acc + 1;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    int best = cands[0];
    float best_ms = 0.f;
    mcx_rng r{0x5EEDull, 0, 0, 0};
    for (size_t ci = 0; ci < cands.size() && err == cudaSuccess; ++ci) {
        const int V = cands[ci];
        err = cudaMemcpyAsync(col[0], lat->d_col[0], half, cudaMemcpyDeviceToDevice, ctx->stream);
        if (err == cudaSuccess) err = cudaMemcpyAsync(col[1], lat->d_col[1], half, cudaMemcpyDeviceToDevice, ctx->stream);
        SweepArgs a;
        fill_sweep_args(&a, lat, t, &r);
        a.acc = acc;
        for (int j = 0; j < 3; ++j) a.dst[j] = dst + j;
        const HalfSweepFn fn = pick_half_sweep(lat, alg, V, t);
        const int grid = half_sweep_grid(ctx, fn, lat->W, lat->rows, V);
        const int warm = 2, reps = 8;
        for (int k = 0; k < warm + reps && err == cudaSuccess; ++k) {
            if (k == warm) err = cudaEventRecord(e0, ctx->stream);
            a.sweep = (unsigned long long)(k / 2);
            a.colour = k & 1;
            a.cur = col[a.colour];
            a.oth = col[1 - a.colour];
            fn<<<grid, 256, 0, ctx->stream>>>(a);
            count_launch(ctx);
        }
        if (err == cudaSuccess) err = cudaEventRecord(e1, ctx->stream);
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        if (err == cudaSuccess && (ci == 0 || ms < best_ms)) {
            best_ms = ms;
            best = V;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, scratch, bytes);
    if (err != cudaSuccess) return cuda_fail(err, "autotune");
    lat->tuned_V = best;
    if (chosen) *chosen = best;
    if (ns_per_site) *ns_per_site = (double)best_ms * 1e6 / (8.0 * (double)half);
    return MCX_OK;
}

// after a batched launch: series lengths, counters, the caller's series and counts
static mcx_status batch_tail(mcx_lattice** lats, int n, mcx_rng* rngs, int64_t nsweeps, int64_t** obs_series,
                             mcx_counters* counters) {
    cudaStream_t st = lats[0]->ctx->stream;
    std::vector<unsigned long long> acc(counters ? n : 0);
    for (int i = 0; i < n; ++i) {
        lats[i]->series_len = nsweeps;
        rngs[i].counter += (uint64_t)nsweeps;
        if (obs_series && obs_series[i])
            MCX_CUDA(cudaMemcpyAsync(obs_series[i], lats[i]->d_series, (size_t)nsweeps * 3 * sizeof(int64_t),
                                     cudaMemcpyDeviceToHost, st));
        if (counters)
            MCX_CUDA(cudaMemcpyAsync(&acc[i], lats[i]->d_acc, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    }
    MCX_CUDA(cudaStreamSynchronize(st));  // acc outlives the copies
    if (counters)
        for (int i = 0; i < n; ++i) {
            counters[i].attempts += (uint64_t)lats[i]->N * (uint64_t)nsweeps;
            counters[i].accepted += acc[i];
        }
    return MCX_OK;
}

extern "C" MCX_API mcx_status mcx_sweep_batch(mcx_lattice** lats, int32_t n, mcx_algorithm alg, const double* betas,
                                              mcx_rng* rngs, int64_t nsweeps, int64_t** obs_series,
                                              mcx_counters* counters) {
    if (!lats || !betas || !rngs || n < 1) return fail(MCX_ERR_INVALID_ARG, "NULL argument or no lattice");
    if (nsweeps < 0) return fail(MCX_ERR_INVALID_ARG, "nsweeps < 0");
    if (alg != MCX_METROPOLIS && alg != MCX_GLAUBER && alg != MCX_HEATBATH)
        return fail(MCX_ERR_INVALID_ARG, "unknown algorithm %d", (int)alg);
    mcx_ctx* ctx = lats[0] ? lats[0]->ctx : nullptr;
    bool small = true, words = true, fits32 = true;
    std::vector<Table> tabs(n);
    for (int i = 0; i < n; ++i) {
        const mcx_lattice* L = lats[i];
        if (!L) return fail(MCX_ERR_INVALID_ARG, "lattice %d is NULL", i);
        if (L->ctx != ctx) return fail(MCX_ERR_INVALID_ARG, "lattice %d is on another context", i);
        if (L->model != lats[0]->model || L->dim != lats[0]->dim)
            return fail(MCX_ERR_INVALID_ARG, "lattice %d: a batch holds one model and dimension", i);
        if (!std::isfinite(betas[i])) return fail(MCX_ERR_INVALID_ARG, "beta %d must be finite", i);
        if (rngs[i].counter + (uint64_t)nsweeps >= (1ull << 48))
            return fail(MCX_ERR_INVALID_ARG, "sweep counter beyond 2^48");
        MCX_CHECK(build_table(L, alg, betas[i], &tabs[i]));
        small = small && L->layout == MCX_LAYOUT_INT8 && L->N <= kSmallLattice;
        words = words && L->W % 4 == 0;
        fits32 = fits32 && ising_table_fits32(tabs[i].thr, tabs[i].n, 2 * L->dim, alg == MCX_HEATBATH);
    }
    if (nsweeps == 0) return MCX_OK;
    if (n == 1)  // the single-lattice forms
        return mcx_sweep(lats[0], alg, betas[0], &rngs[0], nsweeps, obs_series ? obs_series[0] : nullptr, counters);
    // bit-plane uniforms run one mcx_sweep per lattice (Ising: on the words; Blume-Capel: the
    // batch kernels compile the per-site proposal form in)
    bool planes = false;
    for (int i = 0; i < n; ++i)
        planes = planes || msc_planes_ok(lats[i], alg, tabs[i]) ||
                 (lats[i]->model == MCX_BLUME_CAPEL && lats[i]->uniforms == MCX_UNIFORMS_PLANES && alg != MCX_HEATBATH);
    if (planes) {
        for (int i = 0; i < n; ++i)
            MCX_CHECK(mcx_sweep(lats[i], alg, betas[i], &rngs[i], nsweeps, obs_series ? obs_series[i] : nullptr,
                                counters ? &counters[i] : nullptr));
        return MCX_OK;
    }
    // One cluster per lattice in one launch: medium lattices always; lattices the one-block
    // form also takes (above kClusterMin sites) when the device runs every cluster at once
    // (a few 128^2 chains: 1.5 against 3.6 us per sweep; many chains fill more SMs one block
    // each).  Otherwise one block per lattice, or one call per lattice (identical results).
    bool few = true;
    for (int i = 0; i < n; ++i) few = few && lats[i]->N > kClusterMin;
    if (!small || few) {
        for (int i = 0; i < n; ++i) MCX_CHECK(ensure_series(lats[i], nsweeps));
        bool clustered = false;
        MCX_CHECK(cluster_sweep_batch(lats, n, alg, tabs.data(), rngs, nsweeps, fits32, small, &clustered));
        if (clustered) return batch_tail(lats, n, rngs, nsweeps, obs_series, counters);
    }
    if (!small) {
        for (int i = 0; i < n; ++i)
            MCX_CHECK(mcx_sweep(lats[i], alg, betas[i], &rngs[i], nsweeps, obs_series ? obs_series[i] : nullptr,
                                counters ? &counters[i] : nullptr));
        return MCX_OK;
    }
    std::vector<SmallBatchDesc> descs(n);
    long long maxhalf = 0;
    for (int i = 0; i < n; ++i) {
        mcx_lattice* L = lats[i];
        MCX_CHECK(ensure_series(L, nsweeps));
        SmallBatchDesc& d = descs[i];
        fill_sweep_args(&d.a, L, tabs[i], &rngs[i]);
        d.a.acc = L->d_acc;
        d.a.sweep = rngs[i].counter;
        d.col0 = L->d_col[0];
        d.col1 = L->d_col[1];
        d.half = L->N / 2;
        d.series = reinterpret_cast<long long*>(L->d_series);
        d.state = reinterpret_cast<long long*>(L->d_state);
        maxhalf = std::max(maxhalf, d.half);
    }
    void* scratch = nullptr;
    MCX_CHECK(ctx_scratch(ctx, sizeof(SmallBatchDesc) * (size_t)n, &scratch));
    SmallBatchDesc* d_descs = static_cast<SmallBatchDesc*>(scratch);
    cudaStream_t st = ctx->stream;
    MCX_CUDA(cudaMemcpyAsync(d_descs, descs.data(), sizeof(SmallBatchDesc) * (size_t)n, cudaMemcpyHostToDevice, st));
    const int kind = small_kind(lats[0]->model, words);
    const bool hb = alg == MCX_HEATBATH;
    const bool t32 = kind == 0 && fits32;
    int V = 1;
    if (kind == 0 || kind == 2) {  // the narrowest lattice's width divides every row of the batch
        V = 16;
        for (int i = 0; i < n; ++i) V = std::min(V, small_width(lats[i]->W, lats[i]->N / 2));
    }
    const SmallBatchFn fn = pick_small_fn<BatchK>(lats[0]->dim, hb, kind, t32, V);
    const size_t smem = (size_t)(((maxhalf + 15) & ~15ll) + maxhalf);
    if (smem > 48 * 1024)
        MCX_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fn<<<n, 256, smem, st>>>(d_descs, nsweeps);
    k_prefix_series_batch<<<n, 32, 0, st>>>(d_descs, nsweeps);
    count_launch(ctx, 2);
    MCX_CUDA(cudaGetLastError());
    MCX_CUDA(cudaStreamSynchronize(st));  // the descriptors outlive the copy
    return batch_tail(lats, n, rngs, nsweeps, obs_series, counters);
}

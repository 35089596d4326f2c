// mcx_sweep.cu -- checkerboard half-sweep kernels on the colour-split int8 layout.
//
// One launch updates every site of one colour.  A thread owns V consecutive sites
// of one row (V = 16: one 128-bit load/store per array row; V = 4 when the row is
// not a multiple of 16; V = 1 for rows that are not a multiple of 4).  Neighbour
// sums are formed four sites at a time inside 32-bit words; each Philox4x32-10 call
// feeds the four sites of one word, which is exactly the counter mapping of the
// stream (site i takes word (i>>1)&3 of the call with counter (i>>3, ...)).
//
// Per-sweep energy / magnetisation deltas are reduced per block (warp shuffles)
// and added with one 64-bit atomic per block into the sweep's slot of the series.
#include <cmath>

#include "mcx_device.cuh"
#include "mcx_internal.h"
#include "mcx_sweep.cuh"

namespace mcx {

__device__ __forceinline__ uint32_t upbits(uint32_t w) { return (~w >> 1) & 0x01010101u; }
// per byte: v + 1 for v in {-1, 0, +1}
__device__ __forceinline__ uint32_t plus1(uint32_t w) {
    return ((w & 0x7F7F7F7Fu) + 0x01010101u) & 0x03030303u;
}

template <int V>
__device__ __forceinline__ void load_row(const int8_t* p, uint32_t (&w)[V / 4]) {
    if constexpr (V == 16) {
        const uint4 v = *reinterpret_cast<const uint4*>(p);
        w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
    } else {
        w[0] = *reinterpret_cast<const uint32_t*>(p);
    }
}

template <int V>
__device__ __forceinline__ void store_row(int8_t* p, const uint32_t (&w)[V / 4]) {
    if constexpr (V == 16) {
        *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
    } else {
        *reinterpret_cast<uint32_t*>(p) = w[0];
    }
}

__device__ __forceinline__ int bc_propose(int so, int bit) {
    return bit ? (so == -1 ? 0 : -1) : (so == 1 ? 0 : 1);
}

// Row bookkeeping shared by all kernels: neighbour rows and the in-row parity.
struct RowInfo {
    int p;                   // (y + z + colour) & 1
    long long ryp, rym, rzp, rzm;
};

__device__ __forceinline__ RowInfo row_info(int r, int Ly, int Lz, int colour, int dim) {
    RowInfo ri;
    const int y = r % Ly, z = r / Ly;
    ri.p = (y + z + colour) & 1;
    ri.ryp = (long long)((y + 1 == Ly ? 0 : y + 1) + Ly * z);
    ri.rym = (long long)((y == 0 ? Ly - 1 : y - 1) + Ly * z);
    if (dim == 3) {
        ri.rzp = (long long)(y + Ly * (z + 1 == Lz ? 0 : z + 1));
        ri.rzm = (long long)(y + Ly * (z == 0 ? Lz - 1 : z - 1));
    } else {
        ri.rzp = ri.rzm = 0;
    }
    return ri;
}

// Gathers the V-site word groups of one chunk: own spins and the 2*DIM neighbour
// words, with `side` the in-row neighbour shifted by one site.
template <int DIM, int V>
struct Chunk {
    static constexpr int NW = V / 4;
    uint32_t own[NW];
    uint32_t nb[2 * DIM][NW];

    __device__ __forceinline__ void load(const int8_t* cur, const int8_t* oth, int W, int r, int k0,
                                         const RowInfo& ri) {
        const long long base = (long long)r * W + k0;
        load_row<V>(cur + base, own);
        uint32_t mid[NW];
        load_row<V>(oth + base, mid);
        load_row<V>(oth + ri.ryp * W + k0, nb[1]);
        load_row<V>(oth + ri.rym * W + k0, nb[2]);
        if constexpr (DIM == 3) {
            load_row<V>(oth + ri.rzp * W + k0, nb[4]);
            load_row<V>(oth + ri.rzm * W + k0, nb[5]);
        }
        if (ri.p == 0) {
            const int ke = k0 == 0 ? W - 1 : k0 - 1;
            const uint32_t edge = (uint32_t)(uint8_t)oth[(long long)r * W + ke];
#pragma unroll
            for (int w = 0; w < NW; ++w)
                nb[3][w] = __funnelshift_l(w == 0 ? (edge << 24) : mid[w - 1], mid[w], 8);
        } else {
            const int ke = k0 + V == W ? 0 : k0 + V;
            const uint32_t edge = (uint32_t)(uint8_t)oth[(long long)r * W + ke];
#pragma unroll
            for (int w = 0; w < NW; ++w)
                nb[3][w] = __funnelshift_r(mid[w], w == NW - 1 ? edge : mid[w + 1], 8);
        }
#pragma unroll
        for (int w = 0; w < NW; ++w) nb[0][w] = mid[w];
    }
};

// ------------------------------------------------------------------ Ising --
template <int DIM, int V, bool HB>
__global__ void __launch_bounds__(256) k_ising_cb(const SweepArgs a) {
    constexpr int Z = 2 * DIM;
    constexpr int NT = 2 * (Z + 1);
    constexpr int NW = V / 4;
    __shared__ unsigned long long s_thr[NT];
    for (int t = threadIdx.x; t < NT; t += blockDim.x) s_thr[t] = a.thr[t];
    __syncthreads();
    const int cpr = a.W / V;
    const long long nchunk = (long long)cpr * a.rows;
    const uint32_t w2 = ctr_word2(a.sweep, a.colour, P_ACCEPT);
    int nacc = 0, asum = 0, nup = 0;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nchunk;
         g += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(g / cpr);
        const int k0 = (int)(g - (long long)r * cpr) * V;
        const RowInfo ri = row_info(r, a.Ly, a.Lz, a.colour, DIM);
        Chunk<DIM, V> ch;
        ch.load(a.cur, a.oth, a.W, r, k0, ri);
        const unsigned long long j0 = (unsigned long long)r * a.W + k0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            uint32_t cnt = 0;
#pragma unroll
            for (int d = 0; d < Z; ++d) cnt += upbits(ch.nb[d][w]);
            const uint32_t ob = upbits(ch.own[w]);
            const uint4 rnd = philox10(make_uint4((uint32_t)(j0 >> 2) + w, (uint32_t)a.sweep, w2, a.stream), a.k0, a.k1);
            uint32_t fm = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int n = (cnt >> (8 * b)) & 0xFF;
                const int up = (ob >> (8 * b)) & 1;
                const int al = up ? n : Z - n;
                uint32_t u = b == 0 ? rnd.x : b == 1 ? rnd.y : b == 2 ? rnd.z : rnd.w;
                if (HB && up) u = ~u;
                if ((unsigned long long)u < s_thr[al + (Z + 1) * up]) {
                    fm |= 0xFEu << (8 * b);
                    ++nacc;
                    asum += al;
                    nup += up;
                }
            }
            ch.own[w] ^= fm;
        }
        store_row<V>(a.cur + (long long)r * a.W + k0, ch.own);
    }
    long long v[3] = {2ll * Z * nacc - 4ll * asum, 2ll * nacc - 4ll * nup, (long long)nacc};
    unsigned long long* const dst[3] = {a.dst[0], a.dst[1], a.acc};
    block_add_atomic<3>(v, dst);
}

// One site per thread, for rows whose length is not a multiple of 4.
template <int DIM, bool HB>
__global__ void __launch_bounds__(256) k_ising_cb_site(const SweepArgs a) {
    constexpr int Z = 2 * DIM;
    constexpr int NT = 2 * (Z + 1);
    __shared__ unsigned long long s_thr[NT];
    for (int t = threadIdx.x; t < NT; t += blockDim.x) s_thr[t] = a.thr[t];
    __syncthreads();
    const long long n = (long long)a.W * a.rows;
    const uint32_t w2 = ctr_word2(a.sweep, a.colour, P_ACCEPT);
    int nacc = 0, asum = 0, nup = 0;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
         j += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(j / a.W), k = (int)(j - (long long)r * a.W);
        const RowInfo ri = row_info(r, a.Ly, a.Lz, a.colour, DIM);
        const int s = a.cur[j];
        const int ks = ri.p == 0 ? (k == 0 ? a.W - 1 : k - 1) : (k == a.W - 1 ? 0 : k + 1);
        int S = a.oth[j] + a.oth[(long long)r * a.W + ks] + a.oth[ri.ryp * a.W + k] + a.oth[ri.rym * a.W + k];
        if (DIM == 3) S += a.oth[ri.rzp * a.W + k] + a.oth[ri.rzm * a.W + k];
        const int up = s > 0;
        const int al = (s * S + Z) / 2;
        const uint4 rnd = philox10(make_uint4((uint32_t)(j >> 2), (uint32_t)a.sweep, w2, a.stream), a.k0, a.k1);
        uint32_t u = pick4(rnd, (int)(j & 3));
        if (HB && up) u = ~u;
        if ((unsigned long long)u < s_thr[al + (Z + 1) * up]) {
            a.cur[j] = (int8_t)(-s);
            ++nacc;
            asum += al;
            nup += up;
        }
    }
    long long v[3] = {2ll * Z * nacc - 4ll * asum, 2ll * nacc - 4ll * nup, (long long)nacc};
    unsigned long long* const dst[3] = {a.dst[0], a.dst[1], a.acc};
    block_add_atomic<3>(v, dst);
}

// ------------------------------------------------------------ Blume-Capel --
template <int DIM, int V, bool HB>
__global__ void __launch_bounds__(256) k_bc_cb(const SweepArgs a) {
    constexpr int Z = 2 * DIM;
    constexpr int NC = 2 * Z + 1;
    constexpr int NT = HB ? 2 * NC : 6 * NC;
    constexpr int NW = V / 4;
    __shared__ unsigned long long s_thr[NT];
    for (int t = threadIdx.x; t < NT; t += blockDim.x) s_thr[t] = a.thr[t];
    __syncthreads();
    const int cpr = a.W / V;
    const long long nchunk = (long long)cpr * a.rows;
    const uint32_t w2a = ctr_word2(a.sweep, a.colour, P_ACCEPT);
    const uint32_t w2p = ctr_word2(a.sweep, a.colour, P_PROPOSE);
    int nacc = 0, dP = 0, dM = 0, dQ = 0;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nchunk;
         g += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(g / cpr);
        const int k0 = (int)(g - (long long)r * cpr) * V;
        const RowInfo ri = row_info(r, a.Ly, a.Lz, a.colour, DIM);
        Chunk<DIM, V> ch;
        ch.load(a.cur, a.oth, a.W, r, k0, ri);
        const unsigned long long j0 = (unsigned long long)r * a.W + k0;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
            uint32_t cnt = 0;
#pragma unroll
            for (int d = 0; d < Z; ++d) cnt += plus1(ch.nb[d][w]);
            const uint32_t c0 = (uint32_t)(j0 >> 2) + w;
            const uint4 ra = philox10(make_uint4(c0, (uint32_t)a.sweep, w2a, a.stream), a.k0, a.k1);
            uint4 rp = make_uint4(0, 0, 0, 0);
            if (!HB) rp = philox10(make_uint4(c0, (uint32_t)a.sweep, w2p, a.stream), a.k0, a.k1);
            uint32_t word = ch.own[w];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int S = (cnt >> (8 * b)) & 0xFF;  // c + Z
                const int so = (int)(int8_t)(word >> (8 * b));
                const uint32_t u = b == 0 ? ra.x : b == 1 ? ra.y : b == 2 ? ra.z : ra.w;
                int sn;
                bool acc;
                if (HB) {
                    sn = (unsigned long long)u < s_thr[2 * S] ? -1 : ((unsigned long long)u < s_thr[2 * S + 1] ? 0 : 1);
                    acc = sn != so;
                } else {
                    const uint32_t pw = b == 0 ? rp.x : b == 1 ? rp.y : b == 2 ? rp.z : rp.w;
                    const int bit = (int)(pw >> 31);
                    acc = (unsigned long long)u < s_thr[(so + 1) * 2 * NC + bit * NC + S];
                    sn = bc_propose(so, bit);
                }
                if (acc) {
                    const int ds = sn - so;
                    word = (word & ~(0xFFu << (8 * b))) | ((uint32_t)(uint8_t)(int8_t)sn << (8 * b));
                    ++nacc;
                    dP += ds * (S - Z);
                    dM += ds;
                    dQ += sn * sn - so * so;
                }
            }
            ch.own[w] = word;
        }
        store_row<V>(a.cur + (long long)r * a.W + k0, ch.own);
    }
    long long v[4] = {dP, dM, dQ, nacc};
    unsigned long long* const dst[4] = {a.dst[0], a.dst[1], a.dst[2], a.acc};
    block_add_atomic<4>(v, dst);
}

template <int DIM, bool HB>
__global__ void __launch_bounds__(256) k_bc_cb_site(const SweepArgs a) {
    constexpr int Z = 2 * DIM;
    constexpr int NC = 2 * Z + 1;
    constexpr int NT = HB ? 2 * NC : 6 * NC;
    __shared__ unsigned long long s_thr[NT];
    for (int t = threadIdx.x; t < NT; t += blockDim.x) s_thr[t] = a.thr[t];
    __syncthreads();
    const long long n = (long long)a.W * a.rows;
    const uint32_t w2a = ctr_word2(a.sweep, a.colour, P_ACCEPT);
    const uint32_t w2p = ctr_word2(a.sweep, a.colour, P_PROPOSE);
    int nacc = 0, dP = 0, dM = 0, dQ = 0;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
         j += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(j / a.W), k = (int)(j - (long long)r * a.W);
        const RowInfo ri = row_info(r, a.Ly, a.Lz, a.colour, DIM);
        const int so = a.cur[j];
        const int ks = ri.p == 0 ? (k == 0 ? a.W - 1 : k - 1) : (k == a.W - 1 ? 0 : k + 1);
        int c = a.oth[j] + a.oth[(long long)r * a.W + ks] + a.oth[ri.ryp * a.W + k] + a.oth[ri.rym * a.W + k];
        if (DIM == 3) c += a.oth[ri.rzp * a.W + k] + a.oth[ri.rzm * a.W + k];
        const int S = c + Z;
        const uint32_t u = pick4(philox10(make_uint4((uint32_t)(j >> 2), (uint32_t)a.sweep, w2a, a.stream), a.k0, a.k1), (int)(j & 3));
        int sn;
        bool acc;
        if (HB) {
            sn = (unsigned long long)u < s_thr[2 * S] ? -1 : ((unsigned long long)u < s_thr[2 * S + 1] ? 0 : 1);
            acc = sn != so;
        } else {
            const uint32_t pw = pick4(philox10(make_uint4((uint32_t)(j >> 2), (uint32_t)a.sweep, w2p, a.stream), a.k0, a.k1), (int)(j & 3));
            const int bit = (int)(pw >> 31);
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
    long long v[4] = {dP, dM, dQ, nacc};
    unsigned long long* const dst[4] = {a.dst[0], a.dst[1], a.dst[2], a.acc};
    block_add_atomic<4>(v, dst);
}

// ----------------------------------------------------------- dispatching --
template <int DIM>
static HalfSweepFn pick_kernel_dim(mcx_model model, mcx_algorithm alg, int V) {
    const bool hb = alg == MCX_HEATBATH;
    if (model == MCX_ISING) {
        if (V == 16) return hb ? k_ising_cb<DIM, 16, true> : k_ising_cb<DIM, 16, false>;
        if (V == 4) return hb ? k_ising_cb<DIM, 4, true> : k_ising_cb<DIM, 4, false>;
        return hb ? k_ising_cb_site<DIM, true> : k_ising_cb_site<DIM, false>;
    }
    if (V == 16) return hb ? k_bc_cb<DIM, 16, true> : k_bc_cb<DIM, 16, false>;
    if (V == 4) return hb ? k_bc_cb<DIM, 4, true> : k_bc_cb<DIM, 4, false>;
    return hb ? k_bc_cb_site<DIM, true> : k_bc_cb_site<DIM, false>;
}

HalfSweepFn pick_half_sweep(int dim, mcx_model model, mcx_algorithm alg, int V) {
    return dim == 2 ? pick_kernel_dim<2>(model, alg, V) : pick_kernel_dim<3>(model, alg, V);
}

int vec_width(int64_t W) { return W % 16 == 0 ? 16 : (W % 4 == 0 ? 4 : 1); }

int half_sweep_grid(const mcx_ctx* ctx, int64_t W, int64_t rows, int V) {
    const long long work = (long long)(W / V) * rows;
    long long g = (work + 255) / 256;
    const long long cap = (long long)ctx->num_sms * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

mcx_status build_table(const mcx_lattice* lat, mcx_algorithm alg, double beta, Table* t) {
    if (lat->model == MCX_ISING) return build_ising_table(lat->dim, alg, beta, lat->J, lat->h, t);
    return build_bc_table(lat->dim, alg, beta, lat->J, lat->D, lat->h, t);
}

void fill_sweep_args(SweepArgs* a, const mcx_lattice* lat, const Table& t, const mcx_rng* rng) {
    a->W = (int)lat->W;
    a->Ly = (int)lat->L[1];
    a->Lz = (int)lat->L[2];
    a->rows = (int)lat->rows;
    a->k0 = (uint32_t)rng->seed;
    a->k1 = (uint32_t)(rng->seed >> 32);
    a->stream = rng->stream;
    for (int i = 0; i < t.n; ++i) a->thr[i] = t.thr[i];
}

mcx_status msc_sweep(mcx_lattice* lat, mcx_algorithm alg, const Table& t, const mcx_rng* rng,
                     int64_t nsweeps);  // mcx_msc.cu

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
    MCX_CUDA(cudaMemsetAsync(lat->d_series, 0, (size_t)nsweeps * 3 * sizeof(int64_t), ctx->stream));
    MCX_CUDA(cudaMemsetAsync(lat->d_acc, 0, sizeof(unsigned long long), ctx->stream));
    if (lat->layout == MCX_LAYOUT_MSC64) {
        MCX_CHECK(msc_sweep(lat, alg, t, rng, nsweeps));
    } else {
        SweepArgs a;
        fill_sweep_args(&a, lat, t, rng);
        a.acc = lat->d_acc;
        const int V = vec_width(lat->W);
        const HalfSweepFn fn = pick_half_sweep(lat->dim, lat->model, alg, V);
        const int grid = half_sweep_grid(ctx, lat->W, lat->rows, V);
        for (int64_t s = 0; s < nsweeps; ++s) {
            a.sweep = rng->counter + (uint64_t)s;
            for (int c = 0; c < 2; ++c) {
                a.colour = c;
                a.cur = lat->d_col[c];
                a.oth = lat->d_col[1 - c];
                for (int j = 0; j < 3; ++j) a.dst[j] = (unsigned long long*)(lat->d_series + 3 * s + j);
                fn<<<grid, 256, 0, ctx->stream>>>(a);
            }
        }
        count_launch(ctx, 2 * (uint64_t)nsweeps);
        MCX_CUDA(cudaGetLastError());
    }
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

// mcx_msc.cu -- multi-spin-coded (MSC64) Ising sweeps: 64 same-colour sites per
// uint64 word (bit b of word w of a colour row <-> entry k = 64w + b of the int8
// colour-split layout; bit set = spin up).  Neighbour counts are formed for 64
// sites at once with bit-sliced adders.  With per-site uniforms every site draws its
// own Philox word, so results are bit-identical to the int8 kernels, and only rules in
// the rank or the class form of k_msc_metro (Metropolis or Glauber without a field) are
// swept on the words: the other rules (heat bath, a field) would need a per-site table
// lookup, which on a GB300 ran at 451-479 attempts/ns against 749-759 on the int8 words, so
// MSC64 lattices sweep those on their int8 arrays (mcx_sweep unpacks before and packs after
// the call).
// With bit-plane uniforms (mcx_lattice_set_uniforms) every Ising rule is swept on the
// words, in the rank, class or general form of k_msc_metro.
#include "mcx_device.cuh"
#include "mcx_internal.h"
#include "mcx_sweep.cuh"

namespace mcx {

struct MscArgs {
    unsigned long long* cur;
    const unsigned long long* oth;
    int nw;  // words per row
    int W, Ly, Lz, rows, colour;
    int nw_shift, ly_shift;  // log2 of nw / Ly when they are powers of two, else -1
    uint32_t pmask[8][7];    // bit-plane uniforms: all ones where bit 31-p of class k's threshold is set
    // the general form: per class c = aligned count + (Z+1) * (spin up), all ones where bit
    // 31-p of its threshold is set / where it always flips; the low 24 bits of its threshold
    uint32_t gmask[8][14], galways[14], gt24[14];
    int hb;  // heat bath: up spins compare the complement of u
    uint32_t k0, k1, stream;
    unsigned long long sweep;
    unsigned long long* dst[2];
    unsigned long long* acc;
    unsigned long long thr[14];
};

__global__ void k_msc_pack(const int8_t* __restrict__ col, unsigned long long* __restrict__ msc,
                           long long nwords) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nwords;
         q += (long long)gridDim.x * blockDim.x) {
        const uint4* p = reinterpret_cast<const uint4*>(col + q * 64);
        unsigned long long word = 0;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const uint4 x = p[v];
            const uint32_t xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int b = 0; b < 4; ++b)
                    if (((xs[i] >> (8 * b)) & 0xFF) == 1) word |= 1ull << (16 * v + 4 * i + b);
        }
        msc[q] = word;
    }
}

__global__ void k_msc_unpack(int8_t* __restrict__ col, const unsigned long long* __restrict__ msc,
                             long long nwords) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nwords;
         q += (long long)gridDim.x * blockDim.x) {
        const unsigned long long word = msc[q];
        uint4* p = reinterpret_cast<uint4*>(col + q * 64);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            uint32_t xs[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                uint32_t x = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b)
                    x |= ((word >> (16 * v + 4 * i + b)) & 1ull ? 0x01u : 0xFFu) << (8 * b);
                xs[i] = x;
            }
            p[v] = make_uint4(xs[0], xs[1], xs[2], xs[3]);
        }
    }
}

// Bit-sliced count of set bits over Z words: (b0, b1, b2) with n = b0 + 2 b1 + 4 b2.
template <int Z>
__device__ __forceinline__ void count_bits(const unsigned long long (&x)[Z], unsigned long long& b0,
                                           unsigned long long& b1, unsigned long long& b2) {
    b0 = 0; b1 = 0; b2 = 0;
#pragma unroll
    for (int d = 0; d < Z; ++d) {
        const unsigned long long c0 = b0 & x[d];
        b0 ^= x[d];
        const unsigned long long c1 = b1 & c0;
        b1 ^= c0;
        b2 ^= c1;  // n <= 6 never overflows three bits
    }
}

// k_msc_metro (named for its first rule; FORM selects the rule family): FORM 0, a
// Metropolis-type rule in rank form (no field): every class with at most Z/2 aligned
// neighbours is always accepted, and the threshold t_k of a site with Z/2 + k aligned
// neighbours is the same for both spin states and non-increasing in k.  Aligned
// neighbours are counted bit-sliced (c0, c1, c2) for 64 sites at once; each site's
// uniform is compared with the K = Z/2 thresholds into bit masks A_k (u < t_k), and the
// flips are the always-class sites plus, per class k, the sites whose A_k bit is set.
// PL = false: the per-site Philox word of every other kernel, so results are bit-identical
// to theirs.  PL = true: the bit-plane uniforms (mcx_uniforms PLANES): four Philox blocks
// give planes 0..7 of the 64 sites (bits 31..24 of u), compared with the thresholds bit by
// bit, most significant first, for all 64 sites at once; a site is decided at the first
// plane where its bit and its threshold's differ, and only the sites tied after 8 planes
// (probability 2^-8 each) draw the low 24 bits from a per-site block.
//
// FORM 1: the class form, a threshold below 2^32 for every aligned count, the same for both
// spin states (Glauber without a field); K = Z + 1 classes, none always accepted.  FORM 2 (bit planes only): any Ising rule (heat bath, a field): a site flips iff
// (u ^ x) < t_c for its class c = (aligned count, spin), x all ones for up spins under heat
// bath; the word keeps its eight planes from before the wait, and each plane's per-site
// threshold bit is selected from the class leaves by the bit-sliced count and the spin.
template <int DIM, bool PL, int FORM>
__global__ void __launch_bounds__(288, 3) k_msc_metro(const MscArgs a) {
    static_assert(PL || FORM != 2, "the general form is swept with bit-plane uniforms only");
    constexpr bool ALL = FORM == 1, GEN = FORM == 2;
    constexpr int Z = 2 * DIM;
    constexpr int K = GEN ? 1 : ALL ? Z + 1 : Z / 2;
    constexpr int A0 = ALL ? 0 : Z / 2 + 1;  // aligned count of class 0
    uint32_t tk[K];
#pragma unroll
    for (int k = 0; k < K; ++k) tk[k] = (uint32_t)a.thr[A0 + k];  // < 2^32 for these classes
    pdl_trigger();
    const int nwords = a.nw * a.rows;  // < 2^28 words (N <= 2^34 sites)
    const PhiloxPre pre = philox_pre((uint32_t)a.sweep, ctr_word2(a.sweep, a.colour, PL ? P_PLANES : P_ACCEPT), a.k0);
    const PhiloxPre pre_tail = philox_pre((uint32_t)a.sweep, ctr_word2(a.sweep, a.colour, P_TAIL), a.k0);
    // a thread's counts fit 32 bits: at most 64 * 6 per word, ceil(2^27 / 131,328) words
    uint32_t nacc = 0, asum = 0, nup = 0;
    // every block takes an equal contiguous range of words (with 3 blocks per SM 2 % faster
    // on a GB300 than the grid-stride walk; 2 or 4 blocks per SM were slower either way);
    // 288 threads per block give the 131,072 words of a 4096^2 or 256^3 colour one word per
    // thread (256 left 31 threads of each block a second word: 3-8 % slower)
    const int gb = (int)((long long)blockIdx.x * nwords / gridDim.x);
    const int ge = (int)((long long)(blockIdx.x + 1) * nwords / gridDim.x);
    // The uniforms of a word do not depend on the lattice (its 64 sites start at colour index
    // 64 g, so its Philox counters start at 16 g), nor do its neighbours' addresses: each
    // word's draws, their comparisons with every class threshold (lt[k]: u < t_k; with bit
    // planes eq[k]: the top 8 bits of u equal those of t_k) and its load indices are done
    // before the word's loads -- for the first word before the wait for the previous
    // half-sweep.  (The tails of the sites tied with some threshold drawn there too, before
    // the class masks are known, ran slower: 2015 against 2040 attempts/ns in 2-D, 1642
    // against 1778 in 3-D.)
    unsigned long long lt[K], eq[K];
    unsigned long long R[GEN ? 8 : 1];  // the general form: planes 0..7 of the word
    int ix_up = 0, ix_dn = 0, ix_side = 0, ix_zp = 0, ix_zm = 0;
    bool shift_left = false;
    auto draw = [&](int g) {
        const uint32_t cbase = 16u * (uint32_t)g;
        if constexpr (GEN) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint4 rnd = philox10_pre(cbase + j, a.stream, pre, a.k0, a.k1);
                R[2 * j] = ((unsigned long long)rnd.y << 32) | rnd.x;
                R[2 * j + 1] = ((unsigned long long)rnd.w << 32) | rnd.z;
            }
        } else if constexpr (PL) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                lt[k] = 0;
                eq[k] = ~0ull;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint4 rnd = philox10_pre(cbase + j, a.stream, pre, a.k0, a.k1);
                const unsigned long long R[2] = {((unsigned long long)rnd.y << 32) | rnd.x,
                                                 ((unsigned long long)rnd.w << 32) | rnd.z};
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int k = 0; k < K; ++k) {  // bit 31 - (2j + h) of t_k, all ones or zero
                        const uint32_t pm = a.pmask[2 * j + h][k];
                        const unsigned long long T = ((unsigned long long)pm << 32) | pm;
                        lt[k] |= eq[k] & T & ~R[h];
                        eq[k] &= ~(T ^ R[h]);
                    }
            }
        } else {
            uint32_t A[K][2];
#pragma unroll
            for (int k = 0; k < K; ++k) A[k][0] = A[k][1] = 0u;
#pragma unroll
            for (int q = 0; q < 16; ++q) {  // 16 Philox blocks of four words
                const uint4 rnd = philox10_pre(cbase + q, a.stream, pre, a.k0, a.k1);
                const uint32_t us[4] = {rnd.x, rnd.y, rnd.z, rnd.w};
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const int j = 4 * q + b;
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        if (us[b] < tk[k]) A[k][j >> 5] |= 1u << (j & 31);
                }
            }
#pragma unroll
            for (int k = 0; k < K; ++k) lt[k] = ((unsigned long long)A[k][1] << 32) | A[k][0];
        }
        const int r = a.nw_shift >= 0 ? g >> a.nw_shift : g / a.nw;
        const int w = g - r * a.nw;
        const int z = DIM == 3 ? (a.ly_shift >= 0 ? r >> a.ly_shift : r / a.Ly) : 0;
        const int y = r - z * a.Ly;
        shift_left = ((y + z + a.colour) & 1) == 0;  // the row's sites sit left of their partners
        ix_up = ((y + 1 == a.Ly ? 0 : y + 1) + a.Ly * z) * a.nw + w;
        ix_dn = ((y == 0 ? a.Ly - 1 : y - 1) + a.Ly * z) * a.nw + w;
        ix_side = r * a.nw + (shift_left ? (w == 0 ? a.nw - 1 : w - 1) : (w == a.nw - 1 ? 0 : w + 1));
        if constexpr (DIM == 3) {
            ix_zp = (y + a.Ly * (z + 1 == a.Lz ? 0 : z + 1)) * a.nw + w;
            ix_zm = (y + a.Ly * (z == 0 ? a.Lz - 1 : z - 1)) * a.nw + w;
        }
    };
    int g = gb + threadIdx.x;
    if (g < ge) draw(g);
    pdl_wait();  // the previous half-sweep's words are complete
    for (; g < ge; g += blockDim.x) {
        const unsigned long long own = a.cur[g];
        unsigned long long al[Z];  // 1 where neighbour d is aligned with the site
        const unsigned long long mid = a.oth[g];
        const unsigned long long side = a.oth[ix_side];
        al[0] = mid;
        al[1] = a.oth[ix_up];
        al[2] = a.oth[ix_dn];
        al[3] = shift_left ? (mid << 1) | (side >> 63) : (mid >> 1) | (side << 63);
        if constexpr (DIM == 3) {
            al[4] = a.oth[ix_zp];
            al[5] = a.oth[ix_zm];
        }
#pragma unroll
        for (int d = 0; d < Z; ++d) al[d] = ~(al[d] ^ own);
        unsigned long long c0, c1, c2;
        count_bits<Z>(al, c0, c1, c2);
        // class masks of A0 + k aligned neighbours (in the rank form the rest always flips)
        unsigned long long m[K];
        unsigned long long flip = 0;
        if constexpr (GEN) {
            // per-site value of a class leaf set: select on the count bits, then on the spin
            auto bc = [](uint32_t x) { return ((unsigned long long)x << 32) | x; };
            auto sel = [](unsigned long long s, unsigned long long x, unsigned long long y) { return (s & x) | (~s & y); };
            auto leaf = [&](const uint32_t* l) {
                auto cnt = [&](const uint32_t* q) {
                    const unsigned long long lo = sel(c1, sel(c0, bc(q[3]), bc(q[2])), sel(c0, bc(q[1]), bc(q[0])));
                    if constexpr (DIM == 2) return sel(c2, bc(q[4]), lo);
                    const unsigned long long hi = sel(c1, bc(q[6]), sel(c0, bc(q[5]), bc(q[4])));
                    return sel(c2, hi, lo);
                };
                return sel(own, cnt(l + Z + 1), cnt(l));
            };
            const unsigned long long X = a.hb ? own : 0ull;  // heat bath: up spins compare ~u
            const unsigned long long always = leaf(a.galways);
            unsigned long long less = 0, tied = ~always;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const unsigned long long T = leaf(a.gmask[q]), Re = R[q] ^ X;
                less |= tied & T & ~Re;
                tied &= ~(T ^ Re);
            }
            flip = always | less;
            while (tied) {  // top 8 bits equal to the class threshold's: compare the low 24
                const int b = __ffsll((long long)tied) - 1;
                tied &= tied - 1;
                const uint4 rr = philox10_pre(16u * (uint32_t)g + (uint32_t)(b >> 2), a.stream, pre_tail, a.k0, a.k1);
                const int up = (int)((own >> b) & 1ull);
                const int cls = (int)((c0 >> b) & 1ull) + 2 * (int)((c1 >> b) & 1ull) + 4 * (int)((c2 >> b) & 1ull) +
                                (Z + 1) * up;
                const uint32_t lo = (pick4(rr, b & 3) & 0xFFFFFFu) ^ ((a.hb && up) ? 0xFFFFFFu : 0u);
                if (lo < a.gt24[cls]) flip |= 1ull << b;
            }
        } else if constexpr (ALL) {
#pragma unroll
            for (int k = 0; k < K; ++k) m[k] = (k & 1 ? c0 : ~c0) & (k & 2 ? c1 : ~c1) & (k & 4 ? c2 : ~c2);
        } else if constexpr (DIM == 2) {
            m[0] = c0 & c1;  // 3 = 011
            m[1] = c2;       // 4 = 100
            flip = ~(m[0] | m[1]);
        } else {
            m[0] = c2 & ~c1 & ~c0;  // 4 = 100
            m[1] = c2 & c0;         // 5 = 101
            m[2] = c2 & c1;         // 6 = 110
            flip = ~c2;
        }
        if constexpr (!GEN) {
#pragma unroll
            for (int k = 0; k < K; ++k) flip |= m[k] & lt[k];
        }
        if constexpr (PL && !GEN) {
            unsigned long long tied = 0;  // top 8 bits equal to the class threshold's
#pragma unroll
            for (int k = 0; k < K; ++k) tied |= m[k] & eq[k];
            while (tied) {  // compare the low 24 bits
                const int b = __ffsll((long long)tied) - 1;
                tied &= tied - 1;
                const uint4 rr = philox10_pre(16u * (uint32_t)g + (uint32_t)(b >> 2), a.stream, pre_tail, a.k0, a.k1);
                uint32_t t24 = 0;
#pragma unroll
                for (int k = 0; k < K; ++k)
                    if ((m[k] >> b) & 1ull) t24 = tk[k] & 0xFFFFFFu;
                if ((pick4(rr, b & 3) & 0xFFFFFFu) < t24) flip |= 1ull << b;
            }
        }
        a.cur[g] = own ^ flip;
        nacc += __popcll(flip);
        nup += __popcll(flip & own);
        asum += __popcll(flip & c0) + 2u * __popcll(flip & c1) + 4u * __popcll(flip & c2);
        if (g + (int)blockDim.x < ge) draw(g + (int)blockDim.x);
    }
    // warp sums by redux (below 2^24), block sums likewise (below 2^29), then one atomic
    // per series entry per block
    __shared__ uint32_t red[3][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t w0 = __reduce_add_sync(0xFFFFFFFFu, nacc), w1 = __reduce_add_sync(0xFFFFFFFFu, asum),
                   w2 = __reduce_add_sync(0xFFFFFFFFu, nup);
    if (lane == 0) {
        red[0][warp] = w0;
        red[1][warp] = w1;
        red[2][warp] = w2;
    }
    __syncthreads();
    if (warp == 0) {
        const bool in = lane < (int)(blockDim.x >> 5);
        const uint32_t n = __reduce_add_sync(0xFFFFFFFFu, in ? red[0][lane] : 0u);
        const uint32_t as = __reduce_add_sync(0xFFFFFFFFu, in ? red[1][lane] : 0u);
        const uint32_t up = __reduce_add_sync(0xFFFFFFFFu, in ? red[2][lane] : 0u);
        if (lane == 0 && n != 0) {
            const long long dP = 2ll * Z * n - 4ll * as, dM = 2ll * n - 4ll * up;
            if (dP != 0) atomicAdd(a.dst[0], (unsigned long long)dP);
            if (dM != 0) atomicAdd(a.dst[1], (unsigned long long)dM);
            atomicAdd(a.acc, (unsigned long long)n);
        }
    }
}

// Whether a table has the rank form of k_msc_metro: always for <= Z/2 aligned
// neighbours, equal for both spin states above, non-increasing in the aligned count.
static bool msc_rank_form(const Table& t, int Z) {
    const unsigned long long always = 1ull << 32;
    for (int al = 0; al <= Z; ++al) {
        const unsigned long long dn = t.thr[al], upv = t.thr[al + Z + 1];
        if (al <= Z / 2) {
            if (dn != always || upv != always) return false;
        } else {
            if (dn != upv || dn >= always) return false;
            if (al > Z / 2 + 1 && dn > t.thr[al - 1]) return false;
        }
    }
    return true;
}

// The class form: one threshold below 2^32 per aligned count, equal for both spin states.
static bool msc_class_form(const Table& t, int Z) {
    for (int al = 0; al <= Z; ++al)
        if (t.thr[al] != t.thr[al + Z + 1] || t.thr[al] >= (1ull << 32)) return false;
    return true;
}

// Whether `alg` with table `t` is swept on the packed words with per-site uniforms: the rank
// form of k_msc_metro (Metropolis without a field) or its class form (Glauber without a
// field: each site's word compared with all z+1 class thresholds).
bool msc_rank_ok(const mcx_lattice* lat, mcx_algorithm alg, const Table& t) {
    return lat->model == MCX_ISING && alg != MCX_HEATBATH &&
           (msc_rank_form(t, 2 * lat->dim) || msc_class_form(t, 2 * lat->dim));
}

// Whether a call of `alg` on `lat` draws bit-plane uniforms (and so runs on the packed words):
// every Ising rule does once the lattice asks for them (rank, class or general form).
bool msc_planes_ok(const mcx_lattice* lat, mcx_algorithm, const Table&) {
    return lat->uniforms == MCX_UNIFORMS_PLANES && lat->model == MCX_ISING;
}

// Whether a multi-sweep call on an int8 Ising lattice may run on a transient MSC64 copy
// (packed at the start of the call, unpacked at its end): a rule in the rank or the class form
// of k_msc_metro, rows of a multiple of 64 same-colour sites.  Same stream, same
// results; the copy is allocated on first use (within the HBM budget, else the call
// stays on the int8 kernels).
// Allocates the transient copy once (MCX_OK, MCX_ERR_BUDGET or MCX_ERR_OOM; sets no error).
static mcx_status msc_copy_alloc(mcx_lattice* lat) {
    if (lat->d_msc[0]) return MCX_OK;
    mcx_ctx* ctx = lat->ctx;
    const size_t bytes = (size_t)(lat->N / 2) / 8;
    if (ctx->budget && ctx->used + 2 * bytes > ctx->budget) return MCX_ERR_BUDGET;
    void* p0 = nullptr;
    void* p1 = nullptr;
    if (cudaMalloc(&p0, bytes) != cudaSuccess || cudaMalloc(&p1, bytes) != cudaSuccess) {
        cudaGetLastError();  // a failed allocation leaves no sticky error
        if (p0) cudaFree(p0);
        return MCX_ERR_OOM;
    }
    ctx->used += 2 * bytes;
    lat->device_bytes += (int64_t)(2 * bytes);
    lat->d_msc[0] = (unsigned long long*)p0;
    lat->d_msc[1] = (unsigned long long*)p1;
    return MCX_OK;
}

bool msc_transient_ok(mcx_lattice* lat, mcx_algorithm alg, const Table& t) {
    if (lat->layout != MCX_LAYOUT_INT8 || !lat->allow_packing || lat->L[0] % 128 != 0 || !msc_rank_ok(lat, alg, t))
        return false;
    return msc_copy_alloc(lat) == MCX_OK;  // else the call stays on the int8 kernels
}

// The transient copy that a rank-form call with bit-plane uniforms of an int8 lattice
// must run on (the int8 kernels draw per-site words only).
mcx_status msc_planes_copy(mcx_lattice* lat) {
    if (!lat->allow_packing)
        return fail(MCX_ERR_INVALID_ARG, "bit-plane uniforms sweep the packed copy, and packing is off");
    const mcx_status st = msc_copy_alloc(lat);
    if (st != MCX_OK)
        return fail(st, "bit-plane uniforms: no room for the packed copy (%lld bytes)", (long long)(lat->N / 8));
    return MCX_OK;
}

static int grid_cap(const mcx_ctx* ctx, long long work) {
    long long g = (work + 255) / 256;
    const long long cap = (long long)ctx->num_sms * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

mcx_status msc_pack(mcx_lattice* lat) {
    mcx_ctx* ctx = lat->ctx;
    const long long nwords = lat->N / 2 / 64;
    for (int c = 0; c < 2; ++c)
        k_msc_pack<<<grid_cap(ctx, nwords), 256, 0, ctx->stream>>>(lat->d_col[c], lat->d_msc[c], nwords);
    count_launch(ctx, 2);
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

mcx_status msc_unpack(mcx_lattice* lat) {
    mcx_ctx* ctx = lat->ctx;
    const long long nwords = lat->N / 2 / 64;
    for (int c = 0; c < 2; ++c)
        k_msc_unpack<<<grid_cap(ctx, nwords), 256, 0, ctx->stream>>>(lat->d_col[c], lat->d_msc[c], nwords);
    count_launch(ctx, 2);
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

// `nsweeps` sweeps of the packed words with k_msc_metro (the caller checked msc_rank_ok).
mcx_status msc_sweep(mcx_lattice* lat, mcx_algorithm alg, const Table& t, const mcx_rng* rng, int64_t nsweeps) {
    mcx_ctx* ctx = lat->ctx;
    MscArgs a;
    a.nw = (int)(lat->W / 64);
    a.W = (int)lat->W;
    a.Ly = (int)lat->L[1];
    a.Lz = (int)lat->L[2];
    a.rows = (int)lat->rows;
    a.k0 = (uint32_t)rng->seed;
    a.k1 = (uint32_t)(rng->seed >> 32);
    a.stream = rng->stream;
    a.acc = lat->d_acc;
    for (int i = 0; i < t.n && i < 14; ++i) a.thr[i] = t.thr[i];
    auto log2_or = [](long long v) { return v > 0 && (v & (v - 1)) == 0 ? __builtin_ctzll((unsigned long long)v) : -1; };
    a.nw_shift = log2_or(a.nw);
    a.ly_shift = log2_or(a.Ly);
    const int Z = 2 * lat->dim;
    const bool pl = lat->uniforms == MCX_UNIFORMS_PLANES;
    // rank form (any uniforms), else with bit planes the class or the general form
    const int form = msc_rank_form(t, Z) ? 0 : msc_class_form(t, Z) ? 1 : 2;
    const int K = form == 1 ? Z + 1 : Z / 2, A0 = form == 1 ? 0 : Z / 2 + 1;
    for (int p = 0; p < 8; ++p)
        for (int k = 0; k < 7; ++k)
            a.pmask[p][k] = form < 2 && k < K && ((t.thr[A0 + k] >> (31 - p)) & 1ull) ? 0xFFFFFFFFu : 0u;
    for (int c = 0; c < 14; ++c) {
        const unsigned long long v = c < 2 * (Z + 1) ? t.thr[c] : 0;
        for (int p = 0; p < 8; ++p) a.gmask[p][c] = v < (1ull << 32) && ((v >> (31 - p)) & 1ull) ? 0xFFFFFFFFu : 0u;
        a.galways[c] = v >= (1ull << 32) ? 0xFFFFFFFFu : 0u;
        a.gt24[c] = (uint32_t)(v & 0xFFFFFFu);
    }
    a.hb = alg == MCX_HEATBATH;
    using Fn = void (*)(const MscArgs);
    const Fn fns[2][4] = {{k_msc_metro<2, false, 0>, k_msc_metro<2, true, 0>, k_msc_metro<2, true, 1>, k_msc_metro<2, true, 2>},
                          {k_msc_metro<3, false, 0>, k_msc_metro<3, true, 0>, k_msc_metro<3, true, 1>, k_msc_metro<3, true, 2>}};
    const Fn site_fns[2][2] = {{k_msc_metro<2, false, 0>, k_msc_metro<2, false, 1>},
                               {k_msc_metro<3, false, 0>, k_msc_metro<3, false, 1>}};
    const Fn fn = pl ? fns[lat->dim == 3][1 + form] : site_fns[lat->dim == 3][form];  // site: form 0 or 1
    const int grid = occupancy_grid(ctx, (const void*)fn, (long long)a.nw * a.rows, 288, 0);  // one wave
    // every launch after the first depends programmatically on the one before (the
    // kernels read the lattice after pdl_wait)
    cudaLaunchAttribute pdl[1];
    pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    pdl[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(288);
    cfg.stream = ctx->stream;
    cfg.attrs = pdl;
    for (int64_t s = 0; s < nsweeps; ++s) {
        a.sweep = rng->counter + (uint64_t)s;
        for (int c = 0; c < 2; ++c) {
            a.colour = c;
            a.cur = lat->d_msc[c];
            a.oth = lat->d_msc[1 - c];
            a.dst[0] = (unsigned long long*)(lat->d_series + 3 * s);
            a.dst[1] = (unsigned long long*)(lat->d_series + 3 * s + 1);
            cfg.numAttrs = (s == 0 && c == 0) ? 0 : 1;
            MCX_CUDA(cudaLaunchKernelEx(&cfg, fn, a));
        }
    }
    count_launch(ctx, 2 * (uint64_t)nsweeps);
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

}  // namespace mcx

extern "C" MCX_API mcx_status mcx_lattice_set_packing(mcx_lattice* lat, int32_t allow) {
    if (!lat) return mcx::fail(MCX_ERR_INVALID_ARG, "lattice is NULL");
    lat->allow_packing = allow ? 1 : 0;
    return MCX_OK;
}

extern "C" MCX_API mcx_status mcx_lattice_set_uniforms(mcx_lattice* lat, int32_t form) {
    if (!lat) return mcx::fail(MCX_ERR_INVALID_ARG, "lattice is NULL");
    if (form != MCX_UNIFORMS_SITE && form != MCX_UNIFORMS_PLANES)
        return mcx::fail(MCX_ERR_INVALID_ARG, "unknown uniforms form %d", (int)form);
    if (form == MCX_UNIFORMS_PLANES && lat->model == MCX_ISING && lat->L[0] % 128 != 0)
        return mcx::fail(MCX_ERR_INVALID_ARG, "bit-plane uniforms of an Ising lattice need Lx a multiple of 128");
    lat->uniforms = form;
    return MCX_OK;
}

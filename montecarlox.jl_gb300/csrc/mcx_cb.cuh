// mcx_cb.cuh -- device building blocks of the checkerboard kernels, shared by the
// single-lattice sweeps (mcx_sweep.cu) and the batched replica kernels (mcx_pt.cu).
#pragma once

#include <cstdint>

#include "mcx_device.cuh"

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
    } else if constexpr (V == 8) {
        const uint2 v = *reinterpret_cast<const uint2*>(p);
        w[0] = v.x; w[1] = v.y;
    } else {
        w[0] = *reinterpret_cast<const uint32_t*>(p);
    }
}

template <int V>
__device__ __forceinline__ void store_row(int8_t* p, const uint32_t (&w)[V / 4]) {
    if constexpr (V == 16) {
        *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
    } else if constexpr (V == 8) {
        *reinterpret_cast<uint2*>(p) = make_uint2(w[0], w[1]);
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

// Walks the chunks (row y + Ly*z, chunk q of the row) of one colour in grid-stride
// order; the stride is decomposed once, so the loop itself has no divisions.
struct ChunkIter {
    int q, y, z;
    int cpr, Ly, Lz;
    int sq, sy, sz;
    __device__ __forceinline__ ChunkIter(long long g0, long long stride, int cpr_, int Ly_, int Lz_)
        : cpr(cpr_), Ly(Ly_), Lz(Lz_) {
        const long long r0 = g0 / cpr;
        q = (int)(g0 - r0 * cpr);
        y = (int)(r0 % Ly);
        z = (int)(r0 / Ly);
        const long long sr = stride / cpr;
        sq = (int)(stride - sr * cpr);
        sy = (int)(sr % Ly);
        sz = (int)(sr / Ly);
    }
    __device__ __forceinline__ bool valid() const { return z < Lz; }
    __device__ __forceinline__ void next() {
        q += sq;
        int c = 0;
        if (q >= cpr) { q -= cpr; c = 1; }
        y += sy + c;
        c = 0;
        if (y >= Ly) { y -= Ly; c = 1; }
        z += sz + c;
    }
    __device__ __forceinline__ int row() const { return y + Ly * z; }
};

__device__ __forceinline__ RowInfo row_info_yz(int y, int z, int Ly, int Lz, int colour, int dim) {
    RowInfo ri;
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

// Table entry of ising_word: heat-bath entries of up sites (idx >= Z+1) hold 2^32 - thr,
// the probability of staying up; the decision is inverted for up sites once per word,
// so the uniforms need no per-site complement.
__host__ __device__ __forceinline__ unsigned long long ising_tab_entry(unsigned long long thr, int idx, int Z,
                                                                      bool hb) {
    return (hb && idx >= Z + 1) ? (1ull << 32) - thr : thr;
}

// Ising decision for the four sites of one 32-bit word (bytes 0x01 = up, 0xFF = down).
// Per byte: cnt2 = 2 * (down neighbours) from one AND per neighbour word; U1 = 1 for
// an up site; idx2 = 2 * (a + (Z+1)*up) with a = aligned neighbours, which is
// cnt2 for a down site and 2(2Z+1) - cnt2 for an up site, formed byte-parallel with
// (cnt2 ^ 30) = 30 - cnt2 (cnt2 even, <= 12).  4*idx2 is the byte offset of the
// 8-byte table entry (ising_tab_entry form).  One Philox call feeds the four 64-bit
// threshold compares.
// Returns the flip bits (0/1 per byte); accumulates flips, flipped up spins and the
// sum of idx2 over flips (sum a = (isum - (2Z+2)*nup) / 2).
template <int Z, bool HB>
__device__ __forceinline__ uint32_t ising_word(const uint32_t (&nbw)[Z], uint32_t own, uint4 rnd,
                                               const unsigned long long* s_thr, int& nacc, int& nup,
                                               int& isum) {
    uint32_t cnt2 = 0;
#pragma unroll
    for (int d = 0; d < Z; ++d) cnt2 += nbw[d] & 0x02020202u;
    const uint32_t U1 = (~own & 0x02020202u) >> 1;
    const uint32_t idx2 = (cnt2 ^ (U1 * 30u)) - U1 * (uint32_t)(30 - 2 * (2 * Z + 1));
    const uint32_t off = idx2 << 2;
    const char* tb = reinterpret_cast<const char*>(s_thr);
    const uint32_t us[4] = {rnd.x, rnd.y, rnd.z, rnd.w};
    uint32_t fb = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const uint32_t o = __byte_perm(off, 0u, 0x4440u + b);
        const unsigned long long t = *reinterpret_cast<const unsigned long long*>(tb + o);
        if ((unsigned long long)us[b] < t) fb |= 1u << (8 * b);
    }
    // heat bath: an up site's entry is 2^32 - thr, and u below it keeps the spin up
    if (HB) fb ^= U1;
    nacc += __popc(fb);
    nup += __popc(fb & U1);
    isum += (int)(((idx2 & (fb * 0xFFu)) * 0x01010101u) >> 24);
    return fb;
}

// ising_word with 32-bit thresholds: entry t - 1 for the ising_tab_entry value t, usable
// when no entry is 0 (then u < t <=> u <= t - 1 for every t in [1, 2^32]): one 32-bit
// compare per site.  Flip counts go to byte-lane counters of the caller's chunk (at most
// four words: af, au <= 4 and ai <= 4 * 26 per byte), summed once per chunk.
template <int Z, bool HB>
__device__ __forceinline__ uint32_t ising_word32(const uint32_t (&nbw)[Z], uint32_t own, uint4 rnd,
                                                 const uint32_t* s_t32, uint32_t& af, uint32_t& au, uint32_t& ai) {
    uint32_t cnt2 = 0;
#pragma unroll
    for (int d = 0; d < Z; ++d) cnt2 += nbw[d] & 0x02020202u;
    const uint32_t U1 = (~own & 0x02020202u) >> 1;
    const uint32_t idx2 = (cnt2 ^ (U1 * 30u)) - U1 * (uint32_t)(30 - 2 * (2 * Z + 1));
    const uint32_t off = idx2 << 1;  // 4 * idx
    const char* tb = reinterpret_cast<const char*>(s_t32);
    const uint32_t us[4] = {rnd.x, rnd.y, rnd.z, rnd.w};
    uint32_t fb = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const uint32_t o = __byte_perm(off, 0u, 0x4440u + b);
        if (us[b] <= *reinterpret_cast<const uint32_t*>(tb + o)) fb |= 1u << (8 * b);
    }
    if (HB) fb ^= U1;
    af += fb;
    au += fb & U1;
    ai += idx2 & (fb * 0xFFu);
    return fb;
}

// sums of the byte lanes of x (total below 256) and of x with bytes below 256 (any total)
__device__ __forceinline__ int hsum8(uint32_t x) { return (int)((x * 0x01010101u) >> 24); }
__device__ __forceinline__ int hsum16(uint32_t x) {
    x = (x & 0x00FF00FFu) + ((x >> 8) & 0x00FF00FFu);
    return (int)((x * 0x00010001u) >> 16);
}

// Whether every Ising table entry (ising_tab_entry form) is at least 1, so the 32-bit
// form of ising_word32 applies.
inline bool ising_table_fits32(const uint64_t* thr, int n, int Z, bool hb) {
    for (int i = 0; i < n; ++i)
        if (ising_tab_entry(thr[i], i, Z, hb) == 0) return false;
    return true;
}

// Byte-lane counters of a chunk of Blume-Capel words (at most four words: every lane
// stays below 256): plus1 of the new and old spins, their squares, and plus1 times the
// neighbour count cnt = S + Z.
struct BcLanes {
    uint32_t pn = 0, po = 0, qn = 0, qo = 0, cn = 0, co = 0;
};

// The proposal bits of four sites as bytes 0/1: the top bits of the four proposal words
// (the reference's rand(rng, Bool)), or four consecutive bits of a bit plane (the
// multiply copies bit i to bit 8 i; the copies do not overlap).
__device__ __forceinline__ uint32_t bc_site_bits(uint4 rp) {
    const uint32_t txy = __byte_perm(rp.x, rp.y, 0x0073u);  // bytes 0, 1: top bytes of x, y
    const uint32_t tzw = __byte_perm(rp.z, rp.w, 0x0073u);
    return (__byte_perm(txy, tzw, 0x5410u) >> 7) & 0x01010101u;
}
__device__ __forceinline__ uint32_t bc_plane_bits(uint32_t nib) { return (nib * 0x00204081u) & 0x01010101u; }

// Blume-Capel decision for the four sites of one word without per-site branches.
// Metropolis / Glauber: proposal bits as bytes 0/1 (`bits`), table entry (s_old+1)*2*NC + bit*NC + S formed
// byte-parallel, one 64-bit threshold compare per site, the proposed spins and the
// accepted bytes merged with byte masks.  Heat bath: sn = -1 + [u >= T1] + [u >= T12]
// per site from the cumulative thresholds at 2S, 2S+1.  Returns the new word; counts
// changed sites into nacc and the observable deltas into the byte lanes.
template <int Z, bool HB>
__device__ __forceinline__ uint32_t bc_word_swar(const uint32_t (&nbw)[Z], uint32_t own, uint4 ra, uint32_t bits,
                                                 const unsigned long long* s_thr, int& nacc, BcLanes& ln) {
    constexpr int NC = 2 * Z + 1;
    uint32_t cnt = 0;
#pragma unroll
    for (int d = 0; d < Z; ++d) cnt += plus1(nbw[d]);
    const uint32_t po = plus1(own);
    const uint32_t ua[4] = {ra.x, ra.y, ra.z, ra.w};
    const char* tb = reinterpret_cast<const char*>(s_thr);  // 16-byte aligned
    uint32_t nw;
    if (HB) {
        nw = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const uint32_t S = __byte_perm(cnt, 0u, 0x4440u + b);
            const ulonglong2 t = *reinterpret_cast<const ulonglong2*>(tb + 16u * S);  // (T1, T12) at 2S
            const uint32_t c = (uint32_t)((unsigned long long)ua[b] >= t.x) + (uint32_t)((unsigned long long)ua[b] >= t.y);
            nw |= ((c + 0xFFu) & 0xFFu) << (8 * b);
        }
    } else {
        // proposal bits (bytes 0/1), and as 0x00/0xFF masks
        const uint32_t bm = bits * 0xFFu;
        const uint32_t idx = po * (uint32_t)(2 * NC) + bits * (uint32_t)NC + cnt;  // bytes <= 77
        uint32_t f = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const uint32_t e = __byte_perm(idx, 0u, 0x4440u + b);
            if ((unsigned long long)ua[b] < s_thr[e]) f |= 1u << (8 * b);
        }
        const uint32_t am = f * 0xFFu;
        // proposals: bit 0 -> +1 unless the spin is +1 (then 0); bit 1 -> -1 unless it is -1 (then 0)
        const uint32_t is1 = (po >> 1) & 0x01010101u;            // s_old = +1
        const uint32_t ism1 = ~(po | (po >> 1)) & 0x01010101u;  // s_old = -1
        const uint32_t sn0 = 0x01010101u - is1;                  // bytes 0x01 or 0x00
        const uint32_t sn1 = (ism1 ^ 0x01010101u) * 0xFFu;       // bytes 0xFF or 0x00
        const uint32_t sn = (sn1 & bm) | (sn0 & ~bm);
        nw = (sn & am) | (own & ~am);
    }
    const uint32_t x = nw ^ own;  // changed bytes
    nacc += __popc((((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x) & 0x80808080u);
    const uint32_t pn = plus1(nw);
    ln.pn += pn;
    ln.po += po;
    ln.qn += nw & 0x01010101u;
    ln.qo += own & 0x01010101u;
    ln.cn += (cnt & ((pn & 0x01010101u) * 0xFFu)) + ((cnt & (((pn >> 1) & 0x01010101u) * 0xFFu)) << 1);
    ln.co += (cnt & ((po & 0x01010101u) * 0xFFu)) + ((cnt & (((po >> 1) & 0x01010101u) * 0xFFu)) << 1);
    return nw;
}

// Folds a chunk's Blume-Capel byte lanes into (pair, spin, spin2) deltas.
template <int Z>
__device__ __forceinline__ void bc_lanes_fold(const BcLanes& ln, int& dP, int& dM, int& dQ) {
    const int m = hsum8(ln.pn) - hsum8(ln.po);
    dM += m;
    dQ += hsum8(ln.qn) - hsum8(ln.qo);
    dP += (hsum16(ln.cn) - hsum16(ln.co)) - Z * m;
}

// (pair, spin) deltas of a block of Ising flips from the word accumulators
template <int Z>
__device__ __forceinline__ void ising_deltas(int nacc, int nup, int isum, long long& dP, long long& dM) {
    dP = 2ll * Z * nacc - 2ll * ((long long)isum - (2ll * Z + 2) * nup);
    dM = 2ll * nacc - 4ll * nup;
}

}  // namespace mcx

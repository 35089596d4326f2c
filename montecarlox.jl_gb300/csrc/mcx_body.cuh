// mcx_body.cuh -- the per-chunk decisions of the int8 checkerboard kernels, shared by the
// single-lattice launch forms (mcx_sweep.cu: one half-sweep per launch, one block per
// call) and the cluster form (mcx_cluster.cu).  A chunk is V consecutive sites of one
// colour row, already gathered with its neighbour words (Chunk<DIM, V>); the helpers draw
// one Philox4x32-10 call per 4-site word from the chunk's global word index, decide every
// site and leave the new words in ch.own.
#pragma once

#include "mcx_cb.cuh"
#include "mcx_device.cuh"
#include "mcx_sweep.cuh"

namespace mcx {

// Ising tables in the form ising_word / ising_word32 read (entry t - 1 for the T32 form).
template <int DIM, bool HB, bool T32>
__device__ __forceinline__ void ising_tables(const SweepArgs& a, unsigned long long* s_thr, uint32_t* s_t32) {
    constexpr int Z = 2 * DIM;
    constexpr int NT = 2 * (Z + 1);
    for (int t = threadIdx.x; t < NT; t += blockDim.x) {
        const unsigned long long e = ising_tab_entry(a.thr[t], t, Z, HB);
        if (T32) s_t32[t] = (uint32_t)(e - 1);
        else s_thr[t] = e;
    }
}

template <int DIM, bool HB>
__host__ __device__ constexpr int bc_table_size() { return HB ? 2 * (4 * DIM + 1) : 6 * (4 * DIM + 1); }

// One Ising chunk: c0 = global site index of the chunk's first site / 4.  Counts go to
// nacc (flips), nup (flipped up spins) and isum (sum of idx2 over flips).
template <int DIM, int V, bool HB, bool T32>
__device__ __forceinline__ void ising_chunk(Chunk<DIM, V>& ch, uint32_t c0, const SweepKey& key, uint32_t w2,
                                            const unsigned long long* s_thr, const uint32_t* s_t32, int& nacc,
                                            int& nup, int& isum) {
    constexpr int Z = 2 * DIM;
    constexpr int NW = V / 4;
    uint32_t af = 0, au = 0, ai = 0;
    const PhiloxPre pre = philox_pre((uint32_t)key.sweep, w2, key.k0);  // invariant: hoisted out of loops
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        uint32_t nbw[Z];
#pragma unroll
        for (int d = 0; d < Z; ++d) nbw[d] = ch.nb[d][w];
        const uint4 rnd = philox10_pre(c0 + w, key.stream, pre, key.k0, key.k1);
        uint32_t fb;
        if (T32) fb = ising_word32<Z, HB>(nbw, ch.own[w], rnd, s_t32, af, au, ai);
        else fb = ising_word<Z, HB>(nbw, ch.own[w], rnd, s_thr, nacc, nup, isum);
        ch.own[w] ^= fb * 0xFEu;
    }
    if (T32) {
        nacc += hsum8(af);
        nup += hsum8(au);
        isum += hsum16(ai);
    }
}

// One Blume-Capel chunk (acceptance words from one Philox call per four sites; proposal
// bits from the top bits of a second call's words, or with bit planes from one 64-bit
// plane: bit e & 63 of plane e >> 6, planes 2m and 2m+1 being words 0 | 1 << 32 and
// 2 | 3 << 32 of the block at counter m; heat bath needs no proposal).  c0 = e0 / 4 for the
// chunk's first colour index e0 (a chunk of at most 16 aligned sites lies in one plane).
// Deltas go to nacc and (dP, dM, dQ).
// PLM: 0 per-site proposals, 1 plane proposals (both compiled in), 2 as `planes` says.
template <int DIM, int V, bool HB, int PLM = 2>
__device__ __forceinline__ void bc_chunk(Chunk<DIM, V>& ch, uint32_t c0, const SweepKey& key, uint32_t w2a,
                                         uint32_t w2p, bool planes_arg, const unsigned long long* s_thr, int& nacc,
                                         int& dP, int& dM, int& dQ) {
    constexpr int Z = 2 * DIM;
    constexpr int NW = V / 4;
    const bool planes = PLM == 2 ? planes_arg : PLM == 1;
    BcLanes ln;
    unsigned long long plane = 0;
    if (!HB && planes) {
        const unsigned long long e0 = 4ull * c0;
        const uint4 b = philox10(make_uint4((uint32_t)(e0 >> 7), (uint32_t)key.sweep, w2p, key.stream), key.k0, key.k1);
        plane = (e0 >> 6) & 1 ? ((unsigned long long)b.w << 32) | b.z : ((unsigned long long)b.y << 32) | b.x;
    }
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        uint32_t nbw[Z];
#pragma unroll
        for (int d = 0; d < Z; ++d) nbw[d] = ch.nb[d][w];
        const uint4 ra = philox10(make_uint4(c0 + w, (uint32_t)key.sweep, w2a, key.stream), key.k0, key.k1);
        uint32_t bits = 0;
        if (!HB) {
            if (planes)
                bits = bc_plane_bits((uint32_t)(plane >> ((4u * (c0 + w)) & 63u)) & 0xFu);
            else
                bits = bc_site_bits(philox10(make_uint4(c0 + w, (uint32_t)key.sweep, w2p, key.stream), key.k0, key.k1));
        }
        ch.own[w] = bc_word_swar<Z, HB>(nbw, ch.own[w], ra, bits, s_thr, nacc, ln);
    }
    bc_lanes_fold<Z>(ln, dP, dM, dQ);
}

}  // namespace mcx

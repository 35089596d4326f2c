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

// One Blume-Capel chunk (acceptance and proposal words from two Philox calls per word;
// heat bath needs no proposal).  Deltas go to nacc and (dP, dM, dQ).
template <int DIM, int V, bool HB>
__device__ __forceinline__ void bc_chunk(Chunk<DIM, V>& ch, uint32_t c0, const SweepKey& key, uint32_t w2a,
                                         uint32_t w2p, const unsigned long long* s_thr, int& nacc, int& dP, int& dM,
                                         int& dQ) {
    constexpr int Z = 2 * DIM;
    constexpr int NW = V / 4;
    BcLanes ln;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        uint32_t nbw[Z];
#pragma unroll
        for (int d = 0; d < Z; ++d) nbw[d] = ch.nb[d][w];
        const uint4 ra = philox10(make_uint4(c0 + w, (uint32_t)key.sweep, w2a, key.stream), key.k0, key.k1);
        uint4 rp = make_uint4(0, 0, 0, 0);
        if (!HB) rp = philox10(make_uint4(c0 + w, (uint32_t)key.sweep, w2p, key.stream), key.k0, key.k1);
        ch.own[w] = bc_word_swar<Z, HB>(nbw, ch.own[w], ra, rp, s_thr, nacc, ln);
    }
    bc_lanes_fold<Z>(ln, dP, dM, dQ);
}

}  // namespace mcx

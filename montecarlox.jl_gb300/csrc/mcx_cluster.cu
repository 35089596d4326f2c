// mcx_cluster.cu -- every sweep of a call on a medium int8 lattice in one thread-block
// cluster (the sweep loop of SpinSystems' spin_flip! over all sites, ising.jl:25-58 /
// blume_capel.jl:41-85, in checkerboard order, as the other launch forms).
//
// The lattice is cut into units -- rows in 2-D, z-planes in 3-D (the rows a neighbour can
// reach across the cut) -- and CTA k of the cluster owns a contiguous range of units of
// both colours in its shared memory, plus one halo unit on either side.  A half-sweep
// updates the CTA's own units from shared memory only; a thread that updates a chunk of
// its CTA's first or last unit also stores the new words into the halo of the
// neighbouring CTA through distributed shared memory; one cluster barrier ends the
// half-sweep (it orders those stores before the next half-sweep reads them).  Per-sweep
// deltas are summed per warp and added with integer atomics.  The Philox counter of a site
// is its global index, so the results equal the other launch forms bit for bit.
//
// Compared with one launch (or one captured graph node) per half-sweep, which costs
// ~3 us on these sizes, the cluster form pays one hardware barrier of the <= 16 CTAs.
#include <cooperative_groups.h>

#include <algorithm>

#include "mcx_body.cuh"
#include "mcx_internal.h"
#include "mcx_sweep.cuh"

namespace cg = cooperative_groups;

namespace mcx {

namespace {

struct ClusterArgs {
    SweepArgs a;      // geometry, key, table and counter (cur, oth and dst are not used)
    int8_t* g[2];     // the colour arrays in global memory
    long long* series;
    long long nsweeps;
    int units, U;     // units of the cut and rows per unit
};

__device__ __forceinline__ int first_unit(int units, int C, int b) { return (int)((long long)units * b / C); }

template <int KIND, int DIM, int V, bool HB, bool T32>
__global__ void __launch_bounds__(512, 1) k_lattice_cluster(const ClusterArgs ca) {
    extern __shared__ __align__(16) int8_t s_lat[];
    __shared__ __align__(16) unsigned long long s_thr[kMaxTable];
    __shared__ uint32_t s_t32[kMaxTable];
    constexpr int Z = 2 * DIM;
    cg::cluster_group cl = cg::this_cluster();
    const SweepArgs& a0 = ca.a;
    const int C = (int)cl.num_blocks(), k = (int)cl.block_rank();
    const int units = ca.units, U = ca.U, W = a0.W;
    const int u0 = first_unit(units, C, k), nu = first_unit(units, C, k + 1) - u0;
    const int kp = k == 0 ? C - 1 : k - 1, kn = k + 1 == C ? 0 : k + 1;
    const int nu_p = first_unit(units, C, kp + 1) - first_unit(units, C, kp);
    const int unitB = U * W;  // bytes of one unit of one colour (<= 16384)
    const int slab = (((units + C - 1) / C + 2) * unitB + 15) & ~15;
    int8_t* const s[2] = {s_lat, s_lat + slab};
    // own units and both halo units (local unit lu <-> global unit u0 - 1 + lu, cyclic)
    for (int c = 0; c < 2; ++c) {
        const int nwords = (nu + 2) * unitB / 4;
        for (int i = threadIdx.x; i < nwords; i += blockDim.x) {
            const int lu = 4 * i / unitB, off = 4 * i - lu * unitB;
            int gu = u0 - 1 + lu;
            gu = gu < 0 ? gu + units : (gu >= units ? gu - units : gu);
            *reinterpret_cast<uint32_t*>(s[c] + 4 * i) =
                *reinterpret_cast<const uint32_t*>(ca.g[c] + (long long)gu * unitB + off);
        }
    }
    if constexpr (KIND == 0) {
        ising_tables<DIM, HB, T32>(a0, s_thr, s_t32);
    } else {
        for (int t = threadIdx.x; t < kMaxTable; t += blockDim.x) s_thr[t] = a0.thr[t];
    }
    cl.sync();  // every halo is loaded before a neighbour stores into it
    // where this CTA's first unit lives in the previous CTA (its bottom halo) and its last
    // unit in the next CTA (its top halo)
    int8_t* const up0 = cl.map_shared_rank(s[0], kp) + (nu_p + 1) * unitB;
    int8_t* const up1 = cl.map_shared_rank(s[1], kp) + (nu_p + 1) * unitB;
    int8_t* const dn0 = cl.map_shared_rank(s[0], kn);
    int8_t* const dn1 = cl.map_shared_rank(s[1], kn);
    const ChunkIter it0(threadIdx.x, blockDim.x, W / V, U, nu);  // y: row in the unit, z: own unit
    for (long long t = 0; t < ca.nsweeps; ++t) {
        const SweepKey key{a0.sweep + (unsigned long long)t, a0.k0, a0.k1, a0.stream};
        long long v[4] = {0, 0, 0, 0};
        for (int c = 0; c < 2; ++c) {
            int8_t* const cur = c ? s[1] : s[0];  // selects, not a local-memory array
            const int8_t* const oth = c ? s[0] : s[1];
            int8_t* const up_halo = c ? up1 : up0;
            int8_t* const dn_halo = c ? dn1 : dn0;
            const uint32_t w2a = ctr_word2(key.sweep, c, P_ACCEPT), w2p = ctr_word2(key.sweep, c, P_PROPOSE);
            int nacc = 0, nup = 0, isum = 0, dP = 0, dM = 0, dQ = 0;
            for (ChunkIter it = it0; it.valid(); it.next()) {
                const int lu = it.z + 1;
                RowInfo ri;
                int lr;
                long long gr;
                if constexpr (DIM == 2) {  // unit = row: y = u0 + z
                    const int y = u0 + it.z;
                    lr = lu;
                    gr = y;
                    ri.p = (y + c) & 1;
                    ri.ryp = lr + 1;
                    ri.rym = lr - 1;
                    ri.rzp = ri.rzm = 0;
                } else {  // unit = plane: z = u0 + it.z, y wraps inside the plane
                    const int y = it.y, z = u0 + it.z;
                    lr = y + U * lu;
                    gr = y + (long long)U * z;
                    ri.p = (y + z + c) & 1;
                    ri.ryp = (y + 1 == U ? 0 : y + 1) + U * lu;
                    ri.rym = (y == 0 ? U - 1 : y - 1) + U * lu;
                    ri.rzp = y + U * (lu + 1);
                    ri.rzm = y + U * (lu - 1);
                }
                const int k0 = it.q * V;
                Chunk<DIM, V> ch;
                ch.load(cur, oth, W, lr, k0, ri);
                const uint32_t c0 = (uint32_t)(((unsigned long long)gr * W + k0) >> 2);
                if constexpr (KIND == 0) ising_chunk<DIM, V, HB, T32>(ch, c0, key, w2a, s_thr, s_t32, nacc, nup, isum);
                else bc_chunk<DIM, V, HB>(ch, c0, key, w2a, w2p, s_thr, nacc, dP, dM, dQ);
                store_row<V>(cur + lr * W + k0, ch.own);
                const int uoff = it.y * W + k0;
                if (it.z == 0) store_row<V>(up_halo + uoff, ch.own);
                if (it.z == nu - 1) store_row<V>(dn_halo + uoff, ch.own);
            }
            if constexpr (KIND == 0) {
                long long p, m;
                ising_deltas<Z>(nacc, nup, isum, p, m);
                v[0] += p;
                v[1] += m;
            } else {
                v[0] += dP;
                v[1] += dM;
                v[2] += dQ;
            }
            v[3] += nacc;
            cl.sync();  // this colour's own rows and the neighbours' halos are complete
        }
        unsigned long long* const dst[4] = {(unsigned long long*)(ca.series + 3 * t),
                                            (unsigned long long*)(ca.series + 3 * t + 1),
                                            (unsigned long long*)(ca.series + 3 * t + 2), a0.acc};
        warp_add_atomic<4>(v, dst);  // <= 16384 sites of a colour per CTA: < 100 sites per thread and sweep
    }
    // own units back (the last cluster barrier ordered every store into this CTA)
    for (int c = 0; c < 2; ++c) {
        const int nwords = nu * unitB / 4;
        int8_t* const gc = c ? ca.g[1] : ca.g[0];
        const int8_t* const sc = c ? s[1] : s[0];
        for (int i = threadIdx.x; i < nwords; i += blockDim.x)
            *reinterpret_cast<uint32_t*>(gc + (long long)u0 * unitB + 4 * i) =
                *reinterpret_cast<const uint32_t*>(sc + unitB + 4 * i);
    }
}

using ClusterFn = void (*)(const ClusterArgs);

template <int KIND, int DIM, bool HB, bool T32>
ClusterFn pick_cluster_v(int V) {
    if (V == 16) return k_lattice_cluster<KIND, DIM, 16, HB, T32>;
    if (V == 8) return k_lattice_cluster<KIND, DIM, 8, HB, T32>;
    return k_lattice_cluster<KIND, DIM, 4, HB, T32>;
}

template <int DIM>
ClusterFn pick_cluster_dim(bool ising, bool hb, bool t32, int V) {
    if (ising) {
        if (hb) return t32 ? pick_cluster_v<0, DIM, true, true>(V) : pick_cluster_v<0, DIM, true, false>(V);
        return t32 ? pick_cluster_v<0, DIM, false, true>(V) : pick_cluster_v<0, DIM, false, false>(V);
    }
    return hb ? pick_cluster_v<2, DIM, true, false>(V) : pick_cluster_v<2, DIM, false, false>(V);
}

}  // namespace

mcx_status cluster_sweep(mcx_lattice* lat, mcx_algorithm alg, const Table& t, const mcx_rng* rng, int64_t nsweeps,
                         bool* done) {
    *done = false;
    if (lat->layout != MCX_LAYOUT_INT8 || lat->W % 4 != 0 || lat->N > kClusterLattice || nsweeps < 1 ||
        lat->cluster_size < 0)
        return MCX_OK;
    mcx_ctx* ctx = lat->ctx;
    const int units = (int)(lat->dim == 2 ? lat->L[1] : lat->L[2]);
    const int U = (int)(lat->dim == 2 ? 1 : lat->L[1]);
    const long long unitB = (long long)U * lat->W;
    const bool hb = alg == MCX_HEATBATH, ising = lat->model == MCX_ISING;
    const bool t32 = ising && ising_table_fits32(t.thr, t.n, 2 * lat->dim, hb);
    ClusterArgs ca;
    fill_sweep_args(&ca.a, lat, t, rng);
    ca.a.acc = lat->d_acc;
    ca.a.sweep = rng->counter;
    ca.g[0] = lat->d_col[0];
    ca.g[1] = lat->d_col[1];
    ca.series = reinterpret_cast<long long*>(lat->d_series);
    ca.nsweeps = nsweeps;
    ca.units = units;
    ca.U = U;
    // the largest cluster (<= 16 CTAs, one unit each at least) whose CTAs hold at most
    // 16384 sites of a colour and that the device can place
    for (int C = std::min(16, units); C >= 2; --C) {
        const long long per = (long long)((units + C - 1) / C) * unitB;  // own sites of one colour
        if (per > kSmallLattice) break;
        const int V = small_width(lat->W, per);
        const ClusterFn fn = lat->dim == 2 ? pick_cluster_dim<2>(ising, hb, t32, V) : pick_cluster_dim<3>(ising, hb, t32, V);
        const int threads = (int)std::min<long long>(512, std::max<long long>(32, (per / V + 31) & ~31ll));
        const size_t smem = 2 * (size_t)((per + 2 * unitB + 15) & ~15ll);
        if (C > 8) MCX_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        if (smem > 48 * 1024)
            MCX_CUDA(cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3((unsigned)C);
        cfg.blockDim = dim3((unsigned)threads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = ctx->stream;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, (const void*)fn, &cfg) != cudaSuccess || nclusters < 1) {
            (void)cudaGetLastError();
            continue;
        }
        MCX_CUDA(cudaLaunchKernelEx(&cfg, fn, ca));
        count_launch(ctx);
        lat->cluster_size = C;
        *done = true;
        return MCX_OK;
    }
    lat->cluster_size = -1;  // no cluster fits: the per-half-sweep forms
    return MCX_OK;
}

}  // namespace mcx

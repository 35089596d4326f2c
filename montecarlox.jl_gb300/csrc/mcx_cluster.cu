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
    long long* state;  // running (pair, spin, spin2), for the batched prefix
    long long nsweeps;
    int units, U;     // units of the cut and rows per unit
    int zero;         // zero the series slots and the counter first (batched form)
};

__device__ __forceinline__ int first_unit(int units, int C, int b) { return (int)((long long)units * b / C); }

template <int KIND, int DIM, int V, bool HB, bool T32>
__device__ __forceinline__ void cluster_run(const ClusterArgs& ca) {
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
    if (ca.zero) {
        for (long long i = (long long)k * blockDim.x + threadIdx.x; i < 3 * ca.nsweeps; i += (long long)C * blockDim.x)
            ca.series[i] = 0;
        if (k == 0 && threadIdx.x == 0) *a0.acc = 0ull;
    }
    cl.sync();  // every halo is loaded (and the slots zeroed) before a neighbour stores into it
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
            // Blume-Capel: T32 carries the proposal form (bit planes), compiled in
            const uint32_t w2a = ctr_word2(key.sweep, c, P_ACCEPT),
                           w2p = ctr_word2(key.sweep, c, KIND == 2 && T32 ? P_PLANES : P_PROPOSE);
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
                else bc_chunk<DIM, V, HB, T32 ? 1 : 0>(ch, c0, key, w2a, w2p, T32, s_thr, nacc, dP, dM, dQ);
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

template <int KIND, int DIM, int V, bool HB, bool T32>
__global__ void __launch_bounds__(512, 1) k_lattice_cluster(const ClusterArgs ca) {
    cluster_run<KIND, DIM, V, HB, T32>(ca);
}

// Independent lattices (a ParallelChains batch), one cluster each; clusters never wait on
// one another, so the device may run them in any order and number at a time.
template <int KIND, int DIM, int V, bool HB, bool T32>
__global__ void __launch_bounds__(512, 1) k_lattice_cluster_batch(const ClusterArgs* __restrict__ d) {
    cluster_run<KIND, DIM, V, HB, T32>(d[blockIdx.x / cg::this_cluster().num_blocks()]);
}

// the running series of every lattice of a batch (block b: lattice b), as k_prefix_series
__global__ void k_prefix_series_cluster(const ClusterArgs* __restrict__ d, long long n) {
    const ClusterArgs& c = d[blockIdx.x];
    const int j = threadIdx.x;
    if (j >= 3) return;
    long long acc = c.state[j];
    for (long long s = 0; s < n; ++s) {
        acc += c.series[3 * s + j];
        c.series[3 * s + j] = acc;
    }
    c.state[j] = acc;
}

using ClusterFn = void (*)(const ClusterArgs);
using ClusterBatchFn = void (*)(const ClusterArgs*);

template <int KIND, int DIM, int V, bool HB, bool T32>
struct SingleC {
    using Fn = ClusterFn;
    static constexpr Fn fn = k_lattice_cluster<KIND, DIM, V, HB, T32>;
};
template <int KIND, int DIM, int V, bool HB, bool T32>
struct BatchC {
    using Fn = ClusterBatchFn;
    static constexpr Fn fn = k_lattice_cluster_batch<KIND, DIM, V, HB, T32>;
};

template <template <int, int, int, bool, bool> class K, int KIND, int DIM, bool HB, bool T32>
typename K<0, 2, 4, false, false>::Fn pick_cluster_v(int V) {
    if (V == 16) return K<KIND, DIM, 16, HB, T32>::fn;
    if (V == 8) return K<KIND, DIM, 8, HB, T32>::fn;
    return K<KIND, DIM, 4, HB, T32>::fn;
}

template <template <int, int, int, bool, bool> class K, int DIM>
typename K<0, 2, 4, false, false>::Fn pick_cluster_dim(bool ising, bool hb, bool t32, int V) {
    if (ising) {
        if (hb) return t32 ? pick_cluster_v<K, 0, DIM, true, true>(V) : pick_cluster_v<K, 0, DIM, true, false>(V);
        return t32 ? pick_cluster_v<K, 0, DIM, false, true>(V) : pick_cluster_v<K, 0, DIM, false, false>(V);
    }
    // Blume-Capel: t32 selects the bit-plane proposal form (Metropolis / Glauber)
    return hb ? pick_cluster_v<K, 2, DIM, true, false>(V)
              : t32 ? pick_cluster_v<K, 2, DIM, false, true>(V) : pick_cluster_v<K, 2, DIM, false, false>(V);
}

template <template <int, int, int, bool, bool> class K>
typename K<0, 2, 4, false, false>::Fn pick_cluster(int dim, bool ising, bool hb, bool t32, int V) {
    return dim == 2 ? pick_cluster_dim<K, 2>(ising, hb, t32, V) : pick_cluster_dim<K, 3>(ising, hb, t32, V);
}

// The cut of a lattice: units (rows in 2-D, z-planes in 3-D) and rows per unit.
int cut_units(const mcx_lattice* lat) { return (int)(lat->dim == 2 ? lat->L[1] : lat->L[2]); }
int cut_rows(const mcx_lattice* lat) { return (int)(lat->dim == 2 ? 1 : lat->L[1]); }

// own sites of a colour of the largest CTA when the lattice is cut over C CTAs
long long cut_sites(const mcx_lattice* lat, int C) {
    const int units = cut_units(lat);
    return (long long)((units + C - 1) / C) * cut_rows(lat) * lat->W;
}

bool cluster_eligible(const mcx_lattice* lat) {
    return lat->layout == MCX_LAYOUT_INT8 && lat->W % 4 == 0 && lat->N <= kClusterLattice && cut_units(lat) >= 2;
}

void fill_cluster_args(ClusterArgs* ca, mcx_lattice* lat, const Table& t, const mcx_rng* rng, int64_t nsweeps,
                       int zero) {
    fill_sweep_args(&ca->a, lat, t, rng);
    ca->a.acc = lat->d_acc;
    ca->a.sweep = rng->counter;
    ca->g[0] = lat->d_col[0];
    ca->g[1] = lat->d_col[1];
    ca->series = reinterpret_cast<long long*>(lat->d_series);
    ca->state = reinterpret_cast<long long*>(lat->d_state);
    ca->nsweeps = nsweeps;
    ca->units = cut_units(lat);
    ca->U = cut_rows(lat);
    ca->zero = zero;
}

void make_cluster_cfg(int C, int threads, size_t smem, int nclusters, cudaStream_t st, cudaLaunchConfig_t* cfg,
                      cudaLaunchAttribute* attr) {
    *cfg = cudaLaunchConfig_t{};
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg->gridDim = dim3((unsigned)(C * nclusters));
    cfg->blockDim = dim3((unsigned)threads);
    cfg->dynamicSmemBytes = smem;
    cfg->stream = st;
    cfg->attrs = attr;
    cfg->numAttrs = 1;
}

// Launch configuration of `nclusters` clusters of C CTAs; false when the device cannot
// place one such cluster (or, with all_at_once, all of them at the same time).
mcx_status cluster_config(const void* fn, int C, int threads, size_t smem, int nclusters, bool all_at_once,
                          cudaStream_t st, cudaLaunchConfig_t* cfg, cudaLaunchAttribute* attr, bool* ok) {
    if (C > 8) MCX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    if (smem > 48 * 1024) MCX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    make_cluster_cfg(C, threads, smem, nclusters, st, cfg, attr);
    int active = 0;
    *ok = cudaOccupancyMaxActiveClusters(&active, fn, cfg) == cudaSuccess && active >= (all_at_once ? nclusters : 1);
    if (!*ok) (void)cudaGetLastError();
    return MCX_OK;
}

}  // namespace

mcx_status cluster_sweep(mcx_lattice* lat, mcx_algorithm alg, const Table& t, const mcx_rng* rng, int64_t nsweeps,
                         bool* done) {
    *done = false;
    if (!cluster_eligible(lat) || nsweeps < 1 || lat->cluster_size < 0) return MCX_OK;
    const bool hb = alg == MCX_HEATBATH, ising = lat->model == MCX_ISING;
    // Ising: the 32-bit table form; Blume-Capel: bit-plane proposals
    const bool t32 = ising ? ising_table_fits32(t.thr, t.n, 2 * lat->dim, hb)
                           : !hb && lat->uniforms == MCX_UNIFORMS_PLANES;
    const long long unitB = (long long)cut_rows(lat) * lat->W;
    ClusterArgs ca;
    fill_cluster_args(&ca, lat, t, rng, nsweeps, 0);
    const int key = (hb ? 2 : 0) | (t32 ? 1 : 0);
    if (lat->cluster_size > 0 && lat->cluster_key == key) {  // the plan of the previous call
        cudaLaunchConfig_t cfg;
        cudaLaunchAttribute attr[1];
        make_cluster_cfg(lat->cluster_size, lat->cluster_threads, lat->cluster_smem, 1, lat->ctx->stream, &cfg, attr);
        MCX_CUDA(cudaLaunchKernelEx(&cfg, reinterpret_cast<ClusterFn>(const_cast<void*>(lat->cluster_fn)), ca));
        count_launch(lat->ctx);
        *done = true;
        return MCX_OK;
    }
    // the largest cluster (<= 16 CTAs, one unit each at least) whose CTAs hold at most
    // 16384 sites of a colour and that the device can place
    for (int C = std::min(16, cut_units(lat)); C >= 2; --C) {
        const long long per = cut_sites(lat, C);
        if (per > kSmallLattice) break;
        const int V = small_width(lat->W, per);
        const ClusterFn fn = pick_cluster<SingleC>(lat->dim, ising, hb, t32, V);
        const int threads = (int)std::min<long long>(512, std::max<long long>(32, (per / V + 31) & ~31ll));
        const size_t smem = 2 * (size_t)((per + 2 * unitB + 15) & ~15ll);
        cudaLaunchConfig_t cfg;
        cudaLaunchAttribute attr[1];
        bool ok = false;
        MCX_CHECK(cluster_config((const void*)fn, C, threads, smem, 1, false, lat->ctx->stream, &cfg, attr, &ok));
        if (!ok) continue;
        MCX_CUDA(cudaLaunchKernelEx(&cfg, fn, ca));
        count_launch(lat->ctx);
        lat->cluster_size = C;
        lat->cluster_key = key;
        lat->cluster_fn = (const void*)fn;
        lat->cluster_threads = threads;
        lat->cluster_smem = smem;
        *done = true;
        return MCX_OK;
    }
    lat->cluster_size = -1;  // no cluster fits: the per-half-sweep forms
    return MCX_OK;
}

mcx_status cluster_sweep_batch(mcx_lattice** lats, int n, mcx_algorithm alg, const Table* tabs, const mcx_rng* rngs,
                               int64_t nsweeps, bool fits32, bool all_at_once, bool* done) {
    *done = false;
    if (n < 1 || nsweeps < 1) return MCX_OK;
    int cmax = 16;
    for (int i = 0; i < n; ++i) {
        if (!cluster_eligible(lats[i])) return MCX_OK;
        cmax = std::min(cmax, cut_units(lats[i]));
    }
    mcx_lattice* L0 = lats[0];
    mcx_ctx* ctx = L0->ctx;
    const bool hb = alg == MCX_HEATBATH, ising = L0->model == MCX_ISING;
    const bool t32 = ising && fits32;
    // one cluster size for the batch: the largest every lattice takes
    for (int C = cmax; C >= 2; --C) {
        bool fit = true;
        int V = 16;
        long long maxchunks = 0;
        size_t smem = 0;
        for (int i = 0; i < n && fit; ++i) {
            const long long per = cut_sites(lats[i], C);
            fit = per <= kSmallLattice;
            V = std::min(V, small_width(lats[i]->W, per));  // divides every row (powers of two)
            smem = std::max(smem, 2 * (size_t)((per + 2LL * cut_rows(lats[i]) * lats[i]->W + 15) & ~15ll));
        }
        if (!fit) break;
        for (int i = 0; i < n; ++i) maxchunks = std::max(maxchunks, cut_sites(lats[i], C) / V);
        const int threads = (int)std::min<long long>(512, std::max<long long>(32, (maxchunks + 31) & ~31ll));
        const ClusterBatchFn fn = pick_cluster<BatchC>(L0->dim, ising, hb, t32, V);
        cudaLaunchConfig_t cfg;
        cudaLaunchAttribute attr[1];
        bool ok = false;
        MCX_CHECK(cluster_config((const void*)fn, C, threads, smem, n, all_at_once, ctx->stream, &cfg, attr, &ok));
        if (!ok) {
            if (all_at_once) return MCX_OK;  // the one-block batch form instead
            continue;
        }
        std::vector<ClusterArgs> descs(n);
        for (int i = 0; i < n; ++i) fill_cluster_args(&descs[i], lats[i], tabs[i], &rngs[i], nsweeps, 1);
        void* scratch = nullptr;
        MCX_CHECK(ctx_scratch(ctx, sizeof(ClusterArgs) * (size_t)n, &scratch));
        ClusterArgs* d = static_cast<ClusterArgs*>(scratch);
        MCX_CUDA(cudaMemcpyAsync(d, descs.data(), sizeof(ClusterArgs) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
        MCX_CUDA(cudaLaunchKernelEx(&cfg, fn, (const ClusterArgs*)d));
        k_prefix_series_cluster<<<n, 32, 0, ctx->stream>>>(d, nsweeps);
        count_launch(ctx, 2);
        MCX_CUDA(cudaGetLastError());
        MCX_CUDA(cudaStreamSynchronize(ctx->stream));  // the descriptors outlive the copy
        *done = true;
        return MCX_OK;
    }
    return MCX_OK;
}

}  // namespace mcx

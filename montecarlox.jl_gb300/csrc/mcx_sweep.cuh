// mcx_sweep.cuh -- launch arguments of the checkerboard half-sweep kernels.
#pragma once

#include <cstdint>

#include "mcx_internal.h"

namespace mcx {

struct SweepArgs {
    int8_t* cur;        // colour being updated
    const int8_t* oth;  // the other colour
    int W, Ly, Lz, rows, colour;
    uint32_t k0, k1, stream;
    unsigned long long sweep;    // sweep index (added to sweep_base[0] when that is set)
    // device-resident {first sweep index, seed, stream, series offset} that replace
    // (0, k0|k1<<32, stream, 0) when set (captured CUDA graphs), or null; the kernels add
    // the series offset (in sweeps) to their dst slots
    const unsigned long long* sweep_base;
    unsigned long long* dst[3];  // this sweep's (pair, spin, spin2) delta slots
    unsigned long long* acc;     // accepted-move counter
    unsigned long long thr[kMaxTable];
    // Blume-Capel with bit-plane uniforms: proposal bits from bit planes (the block at
    // counter e >> 7 of purpose P_PLANES holds the planes of 128 same-colour sites)
    int planes = 0;
};

struct SweepKey {
    unsigned long long sweep;
    uint32_t k0, k1, stream;
};

#ifdef __CUDACC__
__device__ __forceinline__ SweepKey sweep_key(const SweepArgs& a) {
    if (!a.sweep_base) return SweepKey{a.sweep, a.k0, a.k1, a.stream};
    const unsigned long long seed = a.sweep_base[1];
    return SweepKey{a.sweep_base[0] + a.sweep, (uint32_t)seed, (uint32_t)(seed >> 32), (uint32_t)a.sweep_base[2]};
}

// offset of this sweep's series slots (in int64 entries)
__device__ __forceinline__ unsigned long long series_shift(const SweepArgs& a) {
    return a.sweep_base ? 3ull * a.sweep_base[3] : 0ull;
}
#endif

// captured multi-sweep graphs hold this many sweeps and are replayed back to back
constexpr int64_t kGraphChunk = 64;
// int8 sweep calls of at least this many sweeps may run on a transient MSC64 copy
constexpr int64_t kMscMinSweeps = 16;

using HalfSweepFn = void (*)(const SweepArgs);

// int8 lattices of at most this many sites run all sweeps of a call in one block with
// both colour arrays in shared memory
constexpr long long kSmallLattice = 16384;
// int8 lattices above kClusterMin and up to kClusterLattice sites run all sweeps of a call
// in one thread-block cluster (rows or z-planes spread over its CTAs' shared memory) when
// their rows are a multiple of 4 sites of a colour; per sweep on a GB300: Ising 96^2 2.56 us
// in one block against 1.53 in a cluster, 128^2 3.28 against 1.53; 64^2 1.46 against 1.51;
// 640^2 6.23 with a graph node per half-sweep against 5.58
constexpr long long kClusterMin = 4096;
constexpr long long kClusterLattice = 524288;

// chunk width of the one-block and cluster kernels for rows of W sites of a colour and
// `sites` sites of a colour per block
int small_width(int64_t W, long long sites);
// whether `alg` with table `t` has the rank form swept on 64-sites-per-word words (mcx_msc.cu)
bool msc_rank_ok(const mcx_lattice* lat, mcx_algorithm alg, const Table& t);
// whether a call draws bit-plane uniforms (the lattice asks for them, rank or class form; mcx_msc.cu)
bool msc_planes_ok(const mcx_lattice* lat, mcx_algorithm alg, const Table& t);
// the cluster form; *done = false when it does not apply or no cluster fits the device
mcx_status cluster_sweep(mcx_lattice* lat, mcx_algorithm alg, const Table& t, const mcx_rng* rng, int64_t nsweeps,
                         bool* done);
// independent lattices, one cluster each, in one launch (series zeroed and prefixed on the
// device); fits32: every table has the 32-bit form; all_at_once: only when the device holds
// every cluster of the batch at the same time
mcx_status cluster_sweep_batch(mcx_lattice** lats, int n, mcx_algorithm alg, const Table* tabs, const mcx_rng* rngs,
                               int64_t nsweeps, bool fits32, bool all_at_once, bool* done);

HalfSweepFn pick_half_sweep(const mcx_lattice* lat, mcx_algorithm alg, int V, const Table& t);
int vec_width(int64_t W);
int lattice_width(const mcx_lattice* lat);
int half_sweep_grid(const mcx_ctx* ctx, HalfSweepFn fn, int64_t W, int64_t rows, int V);
int occupancy_grid(const mcx_ctx* ctx, const void* fn, long long work, int block, size_t smem);
mcx_status build_table(const mcx_lattice* lat, mcx_algorithm alg, double beta, Table* t);
void fill_sweep_args(SweepArgs* a, const mcx_lattice* lat, const Table& t, const mcx_rng* rng);

}  // namespace mcx

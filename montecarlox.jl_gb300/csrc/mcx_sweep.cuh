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

using HalfSweepFn = void (*)(const SweepArgs);

// int8 lattices of at most this many sites run all sweeps of a call in one block with
// both colour arrays in shared memory
constexpr long long kSmallLattice = 16384;

HalfSweepFn pick_half_sweep(int dim, mcx_model model, mcx_algorithm alg, int V, const Table& t);
int vec_width(int64_t W);
int lattice_width(const mcx_lattice* lat);
int half_sweep_grid(const mcx_ctx* ctx, HalfSweepFn fn, int64_t W, int64_t rows, int V);
int occupancy_grid(const mcx_ctx* ctx, const void* fn, long long work, int block, size_t smem);
mcx_status build_table(const mcx_lattice* lat, mcx_algorithm alg, double beta, Table* t);
void fill_sweep_args(SweepArgs* a, const mcx_lattice* lat, const Table& t, const mcx_rng* rng);

}  // namespace mcx

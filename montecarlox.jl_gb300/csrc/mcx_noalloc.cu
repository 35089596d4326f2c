// mcx_noalloc.cu -- mcx_sweep_noalloc: the checkerboard sweep of mcx_sweep for
// callers that must not allocate device memory during the call.
//
// Who needs it: code that runs the sweep from inside a loop whose device memory is
// all owned by another allocator -- a Julia program using CUDA.jl's memory pool, a
// PyTorch program using its caching allocator, or a long-running service that
// reserved its HBM up front.  For them a library that calls cudaMalloc/cudaFree on
// its own is a problem: the allocation bypasses the owner's accounting and can fail
// at run time once the pool holds the memory, and cudaFree waits for the whole
// device, stalling every other stream.  mcx_sweep may grow its per-sweep series
// buffer with cudaMalloc/cudaFree; this entry point never does.
//
// Its only scratch -- the per-sweep (pair, spin, spin2) partial sums that the
// half-sweep kernels add into with one atomic per block, plus the accepted-move
// counter -- lives in the file-scope device array g_noalloc_scratch below, of a fixed
// size (kNoallocMaxSweeps sweeps).  Every GPU that loads the library holds that array
// until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "mcx_device.cuh"
#include "mcx_internal.h"
#include "mcx_sweep.cuh"

namespace mcx {

constexpr int64_t kNoallocMaxSweeps = MCX_NOALLOC_MAX_SWEEPS;
constexpr size_t kNoallocWords = (size_t)kNoallocMaxSweeps * 3 + 1;  // partial sums + counter

// The scratch array.  In host code this name is only a stand-in for the device
// object: its device address comes from cudaGetSymbolAddress (noalloc_scratch_ptr).
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoallocWords];

// series[s][j] = state[j] + sum_{s' <= s} partial[s'][j], written to the caller's
// buffer (if any); state := last row; *accepted_out := the counter word.
__global__ void k_noalloc_finish(const long long* partial, long long* series_out, long long* state,
                                 long long n, const unsigned long long* counter,
                                 unsigned long long* accepted_out) {
    const int j = threadIdx.x;
    if (j < 3) {
        long long acc = state[j];
        for (long long s = 0; s < n; ++s) {
            acc += partial[3 * s + j];
            if (series_out) series_out[3 * s + j] = acc;
        }
        state[j] = acc;
    }
    if (j == 3 && accepted_out) *accepted_out = *counter;
}

// Device address of g_noalloc_scratch on `device`, looked up once per device (with
// that device current) and cached for the life of the process.  A device reset
// (cudaDeviceReset, or a primary-context reset by another runtime in the process) may
// reload the module elsewhere; like every other device object of the library, the
// cached address is then invalid and the library must not be used on that device again.
static mcx_status noalloc_scratch_ptr(int device, unsigned long long** out) {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static unsigned long long* cached[kMaxDevices] = {};
    if (device < 0 || device >= kMaxDevices) return fail(MCX_ERR_INVALID_ARG, "device %d unsupported", device);
    std::lock_guard<std::mutex> lock(mu);
    if (!cached[device]) {
        int prev = 0;
        MCX_CUDA(cudaGetDevice(&prev));
        if (prev != device) MCX_CUDA(cudaSetDevice(device));
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (prev != device) cudaSetDevice(prev);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        cached[device] = (unsigned long long*)p;
    }
    *out = cached[device];
    return MCX_OK;
}

}  // namespace mcx

using namespace mcx;

extern "C" MCX_API mcx_status mcx_sweep_noalloc(mcx_lattice* lat, mcx_algorithm alg, double beta, mcx_rng* rng,
                                                int64_t nsweeps, int64_t* obs_series_dev,
                                                uint64_t* accepted_dev) {
    if (!lat || !rng) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (nsweeps < 0) return fail(MCX_ERR_INVALID_ARG, "nsweeps < 0");
    if (nsweeps > kNoallocMaxSweeps)
        return fail(MCX_ERR_INVALID_ARG, "mcx_sweep_noalloc runs at most %lld sweeps per call (got %lld)",
                    (long long)kNoallocMaxSweeps, (long long)nsweeps);
    if (!std::isfinite(beta)) return fail(MCX_ERR_INVALID_ARG, "beta must be finite");
    if (alg != MCX_METROPOLIS && alg != MCX_GLAUBER && alg != MCX_HEATBATH)
        return fail(MCX_ERR_INVALID_ARG, "unknown algorithm %d", (int)alg);
    if (lat->layout != MCX_LAYOUT_INT8) return fail(MCX_ERR_INVALID_ARG, "mcx_sweep_noalloc needs the int8 layout");
    if (rng->counter + (uint64_t)nsweeps >= (1ull << 48))
        return fail(MCX_ERR_INVALID_ARG, "sweep counter beyond 2^48");
    mcx_ctx* ctx = lat->ctx;
    unsigned long long* scratch = nullptr;
    MCX_CHECK(noalloc_scratch_ptr(ctx->device, &scratch));
    unsigned long long* counter = scratch + (size_t)kNoallocMaxSweeps * 3;
    Table t;
    MCX_CHECK(build_table(lat, alg, beta, &t));
    if (msc_planes_ok(lat, alg, t))
        return fail(MCX_ERR_INVALID_ARG, "mcx_sweep_noalloc draws per-site words: bit-plane uniforms need mcx_sweep");
    // the partial sums of this call's sweeps and the counter start at zero
    MCX_CUDA(cudaMemsetAsync(scratch, 0, (size_t)nsweeps * 3 * sizeof(unsigned long long), ctx->stream));
    MCX_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream));
    SweepArgs a;
    fill_sweep_args(&a, lat, t, rng);
    a.acc = counter;
    const int V = vec_width(lat->W);
    const HalfSweepFn fn = pick_half_sweep(lat, alg, V, t);
    const int grid = half_sweep_grid(ctx, fn, lat->W, lat->rows, V);
    for (int64_t s = 0; s < nsweeps; ++s) {
        a.sweep = rng->counter + (uint64_t)s;
        for (int c = 0; c < 2; ++c) {
            a.colour = c;
            a.cur = lat->d_col[c];
            a.oth = lat->d_col[1 - c];
            for (int j = 0; j < 3; ++j) a.dst[j] = scratch + 3 * s + j;
            fn<<<grid, 256, 0, ctx->stream>>>(a);
        }
    }
    k_noalloc_finish<<<1, 32, 0, ctx->stream>>>((const long long*)scratch, (long long*)obs_series_dev,
                                                (long long*)lat->d_state, nsweeps, counter,
                                                (unsigned long long*)accepted_dev);
    count_launch(ctx, 2 * (uint64_t)nsweeps + 1);
    MCX_CUDA(cudaGetLastError());
    rng->counter += (uint64_t)nsweeps;
    // the stored series describes states before these sweeps: report none rather than stale data
    lat->series_len = 0;
    return MCX_OK;
}

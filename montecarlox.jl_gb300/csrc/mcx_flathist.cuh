// mcx_flathist.cuh -- walker descriptors of the flat-histogram kernel, shared with
// the serving loop (which batches Multicanonical jobs of mixed shape).
#pragma once

#include <cstdint>

#include "mcx_internal.h"

struct mcx_flathist {
    mcx_ctx* ctx = nullptr;
    mcx::CtxHold hold;  // keeps ctx alive while this object exists
    int64_t start = 0, step = 1, nbins = 0;
    double* d_lnw = nullptr;
    unsigned long long* d_H = nullptr;
    uint8_t* d_visited = nullptr;
    unsigned long long* d_red = nullptr;  // min, sum, count
};

namespace mcx {

// Per-walker geometry, couplings, binning and schedule (walkers of one launch may
// differ in all of these: the serving loop batches jobs of mixed shape).
struct FHGeom {
    int W, Ly, Lz, dim, model;  // model 0 Ising, 1 Blume-Capel
    long long J, D, h;
    long long start, step, nbins;
    int shift;  // log2(step) if step is a power of two, else -1
    int mode;   // 0 MUCA, 1 Wang-Landau
    double logf;
    long long nsweeps;
    // Wang-Landau with logf = 2^-wl_exp (0 <= wl_exp <= 40): windows whose ln g values are all
    // multiples of 2^-wl_exp below 2^(52 - wl_exp) in magnitude are held as integers in units
    // of logf, so the update ln g -= logf is an integer decrement (the FP64 subtraction of the
    // reference is exact on such values, so the results are the same bits).  0: off.
    int wl_exact;
    int wl_exp;
};

struct FHWalker {
    FHGeom g;
    int8_t* col[2];
    double* lnw;
    unsigned long long* H;
    long long* series;  // [nsweeps][3] or null
    long long* state;   // device (P, M, Q), read at the start and written back at the end, or null
    long long P, M, Q;  // used when state is null; always written back
    unsigned long long steps, accepted;
    unsigned long long sweep0;
    uint32_t k0, k1, stream;
    int status;  // 0 ok, 2 out of range
};

struct FHArgs {
    FHWalker* walkers;
    int nwalkers;
};

// Enqueue one flat-histogram launch over `nwalkers` device walker descriptors (on the
// context's stream, or on `stream`).
mcx_status launch_flathist(mcx_ctx* ctx, FHWalker* d_walkers, int nwalkers);
mcx_status launch_flathist_on(mcx_ctx* ctx, cudaStream_t stream, FHWalker* d_walkers, int nwalkers);
int fh_shift(long long step);
// whether one move's energy change stays well inside the walker's ln g window
bool fh_window_ok(int dim, long long J, long long D, long long h, long long step);

}  // namespace mcx

// mcx_flathist.cu -- Multicanonical and Wang-Landau sweeps (flat-histogram
// importance sampling) for batches of walkers, plus the histogram / weight kernels.
//
// Reference (paths inside MonteCarloX.jl):
//   accept!(alg, x_new, x_old)        src/algorithms/importance_sampling.jl:69-85
//   MUCA record_visit!                src/ensembles/multicanonical.jl:25-30
//   MUCA update!(:simple)             src/ensembles/multicanonical.jl:32-43
//   reset!(::Multicanonical)          src/algorithms/multicanonical.jl:27-33
//   WangLandau accept!                src/algorithms/wang_landau.jl:29-37
//   WangLandauEnsemble update!        src/ensembles/wang_landau.jl:23
//   BinnedObject integer bin index    src/infrastructure/binned_object.jl:22-24
//   merge_histograms! / distribute_logweight!  src/algorithms/parallel_multicanonical.jl:38-73
//
// The acceptance of a site depends on the running total energy and, for
// Wang-Landau, on ln g as modified by the previous attempt, so one walker is
// serial.  Within one colour of a checkerboard sweep, however, every site's energy
// change is fixed in advance (its neighbours are all of the other colour): a warp
// computes 32 proposals, energy changes and log-uniforms in parallel, then lane 0
// runs the short dependent scan over them in site order.  Throughput comes from
// many walkers (one warp each), the pattern of the reference's parallel
// multicanonical walkers.
#include <cmath>
#include <cstring>
#include <vector>

#include "mcx_cb.cuh"
#include "mcx_device.cuh"
#include "mcx_internal.h"
#include "mcx_sweep.cuh"
#include "mcx_flathist.cuh"


namespace mcx {

__device__ __forceinline__ bool fh_bin(long long E, const FHGeom& a, long long& b) {
    const long long x = E - a.start;
    long long q;
    if (a.shift >= 0) q = x >= 0 ? (x >> a.shift) : -((-x) >> a.shift);  // truncating, as Julia div
    else q = x / a.step;
    b = q;
    return q >= 0 && q < a.nbins;
}

constexpr int kFHWarps = 4;

// Each warp keeps a window of kFHWin log-weights around the walker's current bin in
// shared memory, so the serial scan never waits on a global load; the window moves
// when a proposed bin falls outside it (Wang-Landau writes the window back first).
constexpr int kFHWin = 512;
// Bound on |logf(float(U)) - 53 ln 2 (in float) - log(U)|: float(k) is within 2^-24
// relative of k, logf within 1 ulp (<= 2^-18 for results below 64 in magnitude), the
// float constant and subtraction within 2^-18 each: far below 2^-14.
constexpr double kLogMargin = 6.103515625e-05;  // 2^-14

__device__ __forceinline__ long long fh_window_base(long long b, long long nbins) {
    long long wb = b - kFHWin / 2;
    if (wb > nbins - kFHWin) wb = nbins - kFHWin;
    return wb < 0 ? 0 : wb;
}

// FP64 window plus a single-precision copy relative to a centre value c (finite),
// which the serial scan uses to decide without FP64 arithmetic in the common case.
__device__ __forceinline__ void fh_window_load(double* win, float* fwin, const double* lnw, long long wb,
                                               long long nbins, long long centre, int lane, double& c) {
    const double v = lnw[centre];
    c = (v - v == 0.0) ? v : 0.0;  // v finite ? v : 0
    for (int i = lane; i < kFHWin; i += 32) {
        const double x = wb + i < nbins ? lnw[wb + i] : 0.0;
        win[i] = x;
        fwin[i] = (float)(x - c);
    }
    __syncwarp();
}

__device__ __forceinline__ void fh_window_store(const double* win, double* lnw, long long wb, long long nbins, int lane) {
    for (int i = lane; i < kFHWin; i += 32)
        if (wb + i < nbins) lnw[wb + i] = win[i];
    __syncwarp();
}

__global__ void __launch_bounds__(32 * kFHWarps) k_flathist(const FHArgs a) {
    __shared__ long long s_dE[kFHWarps][32];
    __shared__ unsigned long long s_k[kFHWarps][32];  // U = k * 2^-53
    __shared__ float s_lo[kFHWarps][32];              // log(U) lies in [lo, hi]
    __shared__ float s_hi[kFHWarps][32];
    __shared__ double s_win[kFHWarps][kFHWin];
    __shared__ float s_fwin[kFHWarps][kFHWin];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int wid = blockIdx.x * kFHWarps + wl;
    if (wid >= a.nwalkers) return;  // whole warp
    FHWalker& w = a.walkers[wid];
    const FHGeom g = w.g;
    int8_t* const col0 = w.col[0];
    int8_t* const col1 = w.col[1];
    double* const lnw = w.lnw;
    unsigned long long* const H = w.H;
    long long* const series = w.series;
    const uint32_t k0 = w.k0, k1 = w.k1, stream = w.stream;
    const unsigned long long sweep0 = w.sweep0;
    long long P = w.P, M = w.M, Q = w.Q;
    long long E = -g.J * P + g.D * Q - g.h * M;
    long long bo = 0;
    int status = 0;
    if (!fh_bin(E, g, bo)) status = 2;
    double* const win = s_win[wl];
    float* const fwin = s_fwin[wl];
    long long wb = fh_window_base(status ? 0 : bo, g.nbins);
    double cw = 0.0;
    fh_window_load(win, fwin, lnw, wb, g.nbins, status ? 0 : bo, lane, cw);
    float flwo = status ? 0.f : fwin[bo - wb];
    unsigned long long steps = 0, accepted = 0;
    const long long ncol = (long long)g.W * g.Ly * g.Lz;
    const int Z = 2 * g.dim;
    for (long long s = 0; s < g.nsweeps && status == 0; ++s) {
        const unsigned long long t = sweep0 + (unsigned long long)s;
        long long dP = 0, dM = 0, dQ = 0;
        for (int c = 0; c < 2 && status == 0; ++c) {
            int8_t* cur = c ? col1 : col0;
            const int8_t* oth = c ? col0 : col1;
            const uint32_t w2a = ctr_word2(t, c, P_ACCEPT), w2l = ctr_word2(t, c, P_LOW),
                           w2p = ctr_word2(t, c, P_PROPOSE);
            for (long long j0 = 0; j0 < ncol && status == 0; j0 += 32) {
                const long long j = j0 + lane;
                const bool valid = j < ncol;
                int sn = 0, ds = 0, dq = 0, dp = 0;
                long long dE = 0;
                unsigned long long k53 = 0;
                float lo = 0.f, hi = 0.f;
                if (valid) {
                    const int r = (int)(j / g.W), k = (int)(j - (long long)r * g.W);
                    const int y = r % g.Ly, z = r / g.Ly;
                    const RowInfo ri = row_info_yz(y, z, g.Ly, g.Lz, c, g.dim);
                    const int so = cur[j];
                    const int ks = ri.p == 0 ? (k == 0 ? g.W - 1 : k - 1) : (k == g.W - 1 ? 0 : k + 1);
                    int S = oth[j] + oth[(long long)r * g.W + ks] + oth[ri.ryp * g.W + k] + oth[ri.rym * g.W + k];
                    if (Z == 6) S += oth[ri.rzp * g.W + k] + oth[ri.rzm * g.W + k];
                    const uint32_t cj = (uint32_t)(j >> 2);
                    const int lj = (int)(j & 3);
                    if (g.model == 0) sn = -so;
                    else sn = bc_propose(so, (int)(pick4(philox10(make_uint4(cj, (uint32_t)t, w2p, stream), k0, k1), lj) >> 31));
                    ds = sn - so;
                    dq = sn * sn - so * so;
                    dp = ds * S;
                    dE = -g.J * dp + g.D * dq - g.h * ds;
                    const uint32_t whi = pick4(philox10(make_uint4(cj, (uint32_t)t, w2a, stream), k0, k1), lj);
                    const uint32_t wlo = pick4(philox10(make_uint4(cj, (uint32_t)t, w2l, stream), k0, k1), lj);
                    k53 = ((unsigned long long)whi << 21) | (unsigned long long)(wlo >> 11);
                    // single-precision log(U) and a margin that bounds its distance to the
                    // FP64 log of the decision rule (logf: <= 1 ulp, |log U| < 37.5)
                    const float l32 = logf(__ull2float_rn(k53)) - 36.7368005696771f;  // 53 ln 2
                    lo = l32 - (float)kLogMargin;
                    hi = l32 + (float)kLogMargin;
                }
                s_dE[wl][lane] = dE;
                s_k[wl][lane] = k53;
                s_lo[wl][lane] = lo;
                s_hi[wl][lane] = hi;
                __syncwarp();
                unsigned int accmask = 0;
                int i = 0;
                const int n = (int)((ncol - j0) < 32 ? (ncol - j0) : 32);
                for (;;) {
                    long long need = -1;
                    if (lane == 0) {
                        for (; i < n; ++i) {
                            const long long En = E + s_dE[wl][i];
                            long long bn;
                            if (!fh_bin(En, g, bn)) {
                                status = 2;
                                break;
                            }
                            if (bn < wb || bn >= wb + kFHWin) {
                                need = bn;
                                break;
                            }
                            // lr = lnw[bn] - lnw[bo] in FP64, decided from the float copy:
                            // |lr32 - lr| <= 2^-23 (|fa| + |fb| + |lr32|) (two roundings of
                            // the centred values, one of the difference), doubled below
                            const float fa = fwin[bn - wb];
                            const float lr32 = fa - flwo;
                            const float e = (fabsf(fa) + fabsf(flwo) + fabsf(lr32)) * 2.384185791015625e-07f + 1e-30f;
                            bool acc;
                            if (lr32 - e > 0.f || lr32 - e > s_hi[wl][i]) acc = true;
                            else if (lr32 + e <= s_lo[wl][i]) acc = false;
                            else {
                                const double lr = win[bn - wb] - win[bo - wb];
                                acc = (lr > 0.0) ||
                                      (mcx_log((double)s_k[wl][i] * 1.1102230246251565404236316680908203125e-16) < lr);
                            }
                            ++steps;
                            if (acc) {
                                ++accepted;
                                accmask |= 1u << i;
                                E = En;
                                bo = bn;
                                flwo = fa;
                            }
                            if (g.mode == 1) {
                                const double v = win[bo - wb] - g.logf;
                                win[bo - wb] = v;
                                flwo = (float)(v - cw);
                                fwin[bo - wb] = flwo;
                            }
                            atomicAdd(&H[bo], 1ull);
                        }
                    }
                    need = __shfl_sync(0xFFFFFFFFu, need, 0);
                    if (need < 0) break;
                    // move the window around the proposed bin (the current bin stays inside:
                    // one move changes the bin by far less than half the window)
                    __syncwarp();
                    if (g.mode == 1) fh_window_store(win, lnw, wb, g.nbins, lane);
                    const long long bo_all = __shfl_sync(0xFFFFFFFFu, bo, 0);
                    wb = fh_window_base(need, g.nbins);
                    fh_window_load(win, fwin, lnw, wb, g.nbins, need, lane, cw);
                    if (lane == 0) flwo = fwin[bo_all - wb];
                }
                accmask = __shfl_sync(0xFFFFFFFFu, accmask, 0);
                status = __shfl_sync(0xFFFFFFFFu, status, 0);
                if (valid && ((accmask >> lane) & 1u)) {
                    cur[j] = (int8_t)sn;
                    dP += dp;
                    dM += ds;
                    dQ += dq;
                }
                __syncwarp();
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dP += __shfl_down_sync(0xFFFFFFFFu, dP, o);
            dM += __shfl_down_sync(0xFFFFFFFFu, dM, o);
            dQ += __shfl_down_sync(0xFFFFFFFFu, dQ, o);
        }
        if (lane == 0) {
            P += dP;
            M += dM;
            Q += dQ;
            if (status == 0 && series) {
                series[3 * s] = P;
                series[3 * s + 1] = M;
                series[3 * s + 2] = Q;
            }
        }
        P = __shfl_sync(0xFFFFFFFFu, P, 0);
        M = __shfl_sync(0xFFFFFFFFu, M, 0);
        Q = __shfl_sync(0xFFFFFFFFu, Q, 0);
    }
    if (g.mode == 1) fh_window_store(win, lnw, wb, g.nbins, lane);
    if (lane == 0) {
        // a stopped sweep still folds the accepted moves made before the stop
        w.P = P;
        w.M = M;
        w.Q = Q;
        w.steps = steps;
        w.accepted = accepted;
        w.status = status;
    }
}

// lnw[b] -= log(H[b]) for H[b] > 0 (multicanonical.jl:32-43)
__global__ void k_muca_update(double* lnw, const unsigned long long* H, long long n) {
    for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < n;
         b += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h = H[b];
        const double logh = h > 0 ? mcx_log((double)h) : 0.0;
        lnw[b] -= logh;
    }
}

// visited |= H > 0; then min / sum / count of H over the visited bins
__global__ void k_flatness(const unsigned long long* H, uint8_t* visited, long long n, unsigned long long* red) {
    unsigned long long mn = ~0ull, sum = 0, cnt = 0;
    for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < n;
         b += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h = H[b];
        uint8_t v = visited[b];
        if (h > 0 && !v) {
            v = 1;
            visited[b] = 1;
        }
        if (v) {
            mn = h < mn ? h : mn;
            sum += h;
            ++cnt;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long m2 = __shfl_down_sync(0xFFFFFFFFu, mn, o);
        mn = m2 < mn ? m2 : mn;
        sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
        cnt += __shfl_down_sync(0xFFFFFFFFu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (cnt) atomicMin(&red[0], mn);
        atomicAdd(&red[1], sum);
        atomicAdd(&red[2], cnt);
    }
}

__global__ void k_add_hist(unsigned long long* dst, const unsigned long long* src, long long n) {
    for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < n;
         b += (long long)gridDim.x * blockDim.x)
        dst[b] += src[b];
}

mcx_status launch_flathist(mcx_ctx* ctx, FHWalker* d_walkers, int nwalkers) {
    FHArgs a;
    a.walkers = d_walkers;
    a.nwalkers = nwalkers;
    k_flathist<<<(nwalkers + kFHWarps - 1) / kFHWarps, 32 * kFHWarps, 0, ctx->stream>>>(a);
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

bool fh_window_ok(int dim, long long J, long long D, long long h, long long step) {
    const long long z = 2 * dim;
    const long long maxde = 2 * (J < 0 ? -J : J) * z + 2 * (h < 0 ? -h : h) + (D < 0 ? -D : D);
    return maxde / step + 2 < kFHWin / 2;
}

int fh_shift(long long step) {
    for (int sft = 0; sft < 62; ++sft)
        if ((1ll << sft) == step) return sft;
    return -1;
}

static int small_grid(const mcx_ctx* ctx, long long n) {
    long long g = (n + 255) / 256;
    const long long cap = (long long)ctx->num_sms * 8;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace mcx

using namespace mcx;

extern "C" {

MCX_API mcx_status mcx_flathist_destroy(mcx_flathist* fh) {
    if (!fh) return MCX_OK;
    cudaStreamSynchronize(fh->ctx->stream);
    dev_free(fh->ctx, fh->d_lnw, (size_t)fh->nbins * 8);
    dev_free(fh->ctx, fh->d_H, (size_t)fh->nbins * 8);
    dev_free(fh->ctx, fh->d_visited, (size_t)fh->nbins);
    dev_free(fh->ctx, fh->d_red, 3 * 8);
    delete fh;
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_create(mcx_ctx* ctx, int64_t start, int64_t step, int64_t nbins,
                                       mcx_flathist** out) {
    if (!ctx || !out) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (step <= 0 || nbins <= 0) return fail(MCX_ERR_INVALID_ARG, "need step > 0 and nbins > 0");
    mcx_flathist* fh = new mcx_flathist();
    fh->ctx = ctx;
    fh->hold.set(ctx);
    fh->start = start;
    fh->step = step;
    fh->nbins = nbins;
    mcx_status st = dev_alloc(ctx, (void**)&fh->d_lnw, (size_t)nbins * 8);
    if (st == MCX_OK) st = dev_alloc(ctx, (void**)&fh->d_H, (size_t)nbins * 8);
    if (st == MCX_OK) st = dev_alloc(ctx, (void**)&fh->d_visited, (size_t)nbins);
    if (st == MCX_OK) st = dev_alloc(ctx, (void**)&fh->d_red, 3 * 8);
    if (st == MCX_OK) {
        cudaError_t e = cudaMemsetAsync(fh->d_lnw, 0, (size_t)nbins * 8, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(fh->d_H, 0, (size_t)nbins * 8, ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(fh->d_visited, 0, (size_t)nbins, ctx->stream);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMemsetAsync");
    }
    if (st != MCX_OK) {
        mcx_flathist_destroy(fh);
        return st;
    }
    *out = fh;
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_set_logweight(mcx_flathist* fh, const double* host, int64_t n) {
    if (!fh || !host || n != fh->nbins) return fail(MCX_ERR_INVALID_ARG, "expected %lld log-weights", (long long)(fh ? fh->nbins : 0));
    MCX_CUDA(cudaMemcpyAsync(fh->d_lnw, host, (size_t)n * 8, cudaMemcpyHostToDevice, fh->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(fh->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_get_logweight(mcx_flathist* fh, double* host, int64_t n) {
    if (!fh || !host || n != fh->nbins) return fail(MCX_ERR_INVALID_ARG, "expected %lld log-weights", (long long)(fh ? fh->nbins : 0));
    MCX_CUDA(cudaMemcpyAsync(host, fh->d_lnw, (size_t)n * 8, cudaMemcpyDeviceToHost, fh->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(fh->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_set_histogram(mcx_flathist* fh, const int64_t* host, int64_t n) {
    if (!fh || !host || n != fh->nbins) return fail(MCX_ERR_INVALID_ARG, "expected %lld bins", (long long)(fh ? fh->nbins : 0));
    for (int64_t i = 0; i < n; ++i)
        if (host[i] < 0) return fail(MCX_ERR_INVALID_ARG, "histogram counts must be >= 0");
    MCX_CUDA(cudaMemcpyAsync(fh->d_H, host, (size_t)n * 8, cudaMemcpyHostToDevice, fh->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(fh->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_get_histogram(mcx_flathist* fh, int64_t* host, int64_t n) {
    if (!fh || !host || n != fh->nbins) return fail(MCX_ERR_INVALID_ARG, "expected %lld bins", (long long)(fh ? fh->nbins : 0));
    MCX_CUDA(cudaMemcpyAsync(host, fh->d_H, (size_t)n * 8, cudaMemcpyDeviceToHost, fh->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(fh->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_get_visited(mcx_flathist* fh, uint8_t* host, int64_t n) {
    if (!fh || !host || n != fh->nbins) return fail(MCX_ERR_INVALID_ARG, "expected %lld bins", (long long)(fh ? fh->nbins : 0));
    MCX_CUDA(cudaMemcpyAsync(host, fh->d_visited, (size_t)n, cudaMemcpyDeviceToHost, fh->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(fh->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_set_visited(mcx_flathist* fh, const uint8_t* host, int64_t n) {
    if (!fh || !host || n != fh->nbins) return fail(MCX_ERR_INVALID_ARG, "expected %lld bins", (long long)(fh ? fh->nbins : 0));
    for (int64_t i = 0; i < n; ++i)
        if (host[i] > 1) return fail(MCX_ERR_INVALID_ARG, "visited marks are 0 or 1");
    MCX_CUDA(cudaMemcpyAsync(fh->d_visited, host, (size_t)n, cudaMemcpyHostToDevice, fh->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(fh->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_reset(mcx_flathist* fh) {
    if (!fh) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    MCX_CUDA(cudaMemsetAsync(fh->d_H, 0, (size_t)fh->nbins * 8, fh->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_update_muca(mcx_flathist* fh) {
    if (!fh) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    k_muca_update<<<small_grid(fh->ctx, fh->nbins), 256, 0, fh->ctx->stream>>>(fh->d_lnw, fh->d_H, fh->nbins);
    count_launch(fh->ctx);
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_flatness(mcx_flathist* fh, double threshold, int* is_flat, double* ratio) {
    if (!fh) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    unsigned long long init[3] = {~0ull, 0ull, 0ull}, red[3];
    MCX_CUDA(cudaMemcpyAsync(fh->d_red, init, sizeof(init), cudaMemcpyHostToDevice, fh->ctx->stream));
    k_flatness<<<small_grid(fh->ctx, fh->nbins), 256, 0, fh->ctx->stream>>>(fh->d_H, fh->d_visited, fh->nbins, fh->d_red);
    count_launch(fh->ctx);
    MCX_CUDA(cudaGetLastError());
    MCX_CUDA(cudaMemcpyAsync(red, fh->d_red, sizeof(red), cudaMemcpyDeviceToHost, fh->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(fh->ctx->stream));
    double r = 0.0;
    if (red[2] > 0 && red[1] > 0) r = (double)red[0] / ((double)red[1] / (double)red[2]);
    if (ratio) *ratio = r;
    if (is_flat) *is_flat = red[2] > 0 && red[1] > 0 && r >= threshold;
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_merge(mcx_flathist* dst, mcx_flathist* const* src, int nsrc) {
    if (!dst || (nsrc > 0 && !src)) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    for (int i = 0; i < nsrc; ++i) {
        if (!src[i] || src[i]->nbins != dst->nbins) return fail(MCX_ERR_INVALID_ARG, "histogram %d has other bins", i);
        if (src[i] == dst) continue;
        k_add_hist<<<small_grid(dst->ctx, dst->nbins), 256, 0, dst->ctx->stream>>>(dst->d_H, src[i]->d_H, dst->nbins);
        count_launch(dst->ctx);
    }
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_copy_logweight(mcx_flathist* dst, const mcx_flathist* src) {
    if (!dst || !src || src->nbins != dst->nbins) return fail(MCX_ERR_INVALID_ARG, "bad argument");
    MCX_CUDA(cudaMemcpyAsync(dst->d_lnw, src->d_lnw, (size_t)dst->nbins * 8, cudaMemcpyDeviceToDevice, dst->ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_flathist_sweep(mcx_lattice* const* lats, int nwalkers, mcx_flathist* const* fhs, int nfh,
                                      mcx_flathist_mode mode, double logf, mcx_rng* rngs, int64_t nsweeps,
                                      mcx_counters* counters) {
    if (!lats || !fhs || !rngs || nwalkers < 1) return fail(MCX_ERR_INVALID_ARG, "NULL argument or no walkers");
    if (nfh != 1 && nfh != nwalkers) return fail(MCX_ERR_INVALID_ARG, "give one shared histogram or one per walker");
    if (mode != MCX_MUCA && mode != MCX_WANG_LANDAU) return fail(MCX_ERR_INVALID_ARG, "unknown mode");
    if (mode == MCX_WANG_LANDAU && nfh == 1 && nwalkers > 1)
        return fail(MCX_ERR_INVALID_ARG, "Wang-Landau walkers need one log-weight table each");
    if (nsweeps < 0 || !std::isfinite(logf)) return fail(MCX_ERR_INVALID_ARG, "bad nsweeps or logf");
    const mcx_lattice* L0 = lats[0];
    if (!L0) return fail(MCX_ERR_INVALID_ARG, "NULL lattice");
    mcx_ctx* ctx = L0->ctx;
    for (int i = 0; i < nwalkers; ++i) {
        const mcx_lattice* l = lats[i];
        if (!l || l->ctx != ctx || l->model != L0->model || l->dim != L0->dim || l->L[0] != L0->L[0] ||
            l->L[1] != L0->L[1] || l->L[2] != L0->L[2] || l->J != L0->J || l->D != L0->D || l->h != L0->h)
            return fail(MCX_ERR_INVALID_ARG, "walker %d: lattices must share context, model, shape and couplings", i);
        if (l->layout != MCX_LAYOUT_INT8) return fail(MCX_ERR_INVALID_ARG, "walker %d: int8 layout needed", i);
        if (rngs[i].counter + (uint64_t)nsweeps >= (1ull << 48)) return fail(MCX_ERR_INVALID_ARG, "sweep counter beyond 2^48");
    }
    const mcx_flathist* F0 = fhs[0];
    for (int i = 0; i < nfh; ++i)
        if (!fhs[i] || fhs[i]->nbins != F0->nbins || fhs[i]->start != F0->start || fhs[i]->step != F0->step)
            return fail(MCX_ERR_INVALID_ARG, "histograms must share their bins");
    const long long Ji = (long long)L0->J, Di = (long long)L0->D, hi = (long long)L0->h;
    if ((double)Ji != L0->J || (double)Di != L0->D || (double)hi != L0->h)
        return fail(MCX_ERR_INVALID_ARG, "flat-histogram sweeps need integer J, D and h (integer energies)");
    if (!fh_window_ok(L0->dim, Ji, Di, hi, F0->step))
        return fail(MCX_ERR_INVALID_ARG, "one move may change the energy by more than the ln g window holds");
    if (nsweeps == 0) return MCX_OK;
    std::vector<FHWalker> hw(nwalkers);
    for (int i = 0; i < nwalkers; ++i) {
        MCX_CHECK(ensure_series(lats[i], nsweeps));
    }
    // current bookkeeping of every walker
    std::vector<long long> st((size_t)nwalkers * 3);
    for (int i = 0; i < nwalkers; ++i)
        MCX_CUDA(cudaMemcpyAsync(&st[3 * i], lats[i]->d_state, 24, cudaMemcpyDeviceToHost, ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < nwalkers; ++i) {
        FHWalker& w = hw[i];
        std::memset(&w, 0, sizeof(w));
        w.col[0] = lats[i]->d_col[0];
        w.col[1] = lats[i]->d_col[1];
        const mcx_flathist* f = fhs[nfh == 1 ? 0 : i];
        w.lnw = f->d_lnw;
        w.H = f->d_H;
        w.series = (long long*)lats[i]->d_series;
        w.P = st[3 * i];
        w.M = st[3 * i + 1];
        w.Q = st[3 * i + 2];
        w.sweep0 = rngs[i].counter;
        w.k0 = (uint32_t)rngs[i].seed;
        w.k1 = (uint32_t)(rngs[i].seed >> 32);
        w.stream = rngs[i].stream;
    }
    void* dw = nullptr;
    MCX_CHECK(dev_alloc(ctx, &dw, hw.size() * sizeof(FHWalker)));
    FHGeom g;
    std::memset(&g, 0, sizeof(g));
    g.W = (int)L0->W;
    g.Ly = (int)L0->L[1];
    g.Lz = (int)L0->L[2];
    g.dim = L0->dim;
    g.model = L0->model == MCX_ISING ? 0 : 1;
    g.J = Ji;
    g.D = Di;
    g.h = hi;
    g.start = F0->start;
    g.step = F0->step;
    g.nbins = F0->nbins;
    g.shift = fh_shift(F0->step);
    g.mode = mode == MCX_MUCA ? 0 : 1;
    g.logf = logf;
    g.nsweeps = nsweeps;
    for (auto& w : hw) w.g = g;
    cudaError_t e = cudaMemcpyAsync(dw, hw.data(), hw.size() * sizeof(FHWalker), cudaMemcpyHostToDevice, ctx->stream);
    FHArgs a;
    a.walkers = (FHWalker*)dw;
    a.nwalkers = nwalkers;
    if (e == cudaSuccess) {
        k_flathist<<<(nwalkers + kFHWarps - 1) / kFHWarps, 32 * kFHWarps, 0, ctx->stream>>>(a);
        count_launch(ctx);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hw.data(), dw, hw.size() * sizeof(FHWalker), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dev_free(ctx, dw, hw.size() * sizeof(FHWalker));
    if (e != cudaSuccess) return cuda_fail(e, "flat-histogram sweep");
    bool range = false;
    for (int i = 0; i < nwalkers; ++i) {
        const FHWalker& w = hw[i];
        long long s3[3] = {w.P, w.M, w.Q};
        MCX_CUDA(cudaMemcpyAsync(lats[i]->d_state, s3, 24, cudaMemcpyHostToDevice, ctx->stream));
        MCX_CUDA(cudaStreamSynchronize(ctx->stream));
        lats[i]->series_len = w.status ? 0 : nsweeps;
        rngs[i].counter += (uint64_t)nsweeps;
        if (counters) {
            counters[i].attempts += w.steps;
            counters[i].accepted += w.accepted;
        }
        if (w.status) range = true;
    }
    if (range) return fail(MCX_ERR_OUT_OF_RANGE, "an energy left the histogram range (BoundsError)");
    return MCX_OK;
}

}  // extern "C"

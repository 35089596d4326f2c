// mcx_measure.cu -- integrated autocorrelation times of per-sweep series on the device
// (integrated_autocorrelation_time / integrated_autocorrelation_times,
// src/measurements/autocorrelations.jl:28-110), for series held in device memory (the
// lattice, graph and parallel-tempering series) or copied in from the host.
//
// One block per trace.  The block loads the trace (FP64, or a linear combination of up
// to three int64 columns such as -J*pair - h*spin + D*spin2), centres it in a scratch
// array, forms C(0), then walks the lags 32 at a time: warp g of the block sums the
// products c_i c_{i+lag} for i = g (mod 16) with 4 independent FMA chains, lane l taking
// lag = lag0 + l (so a warp reads c_i once, broadcast, and c_{i+lag} as one coalesced
// 256-byte row); the 16 partial sums of a lag are added in a fixed order and thread 0
// applies the reference's truncation -- stop at the first C(t) <= 0 or when
// t > c * tau -- before the next 32 lags are computed.  Sums use FP64 (the reference's
// precision) in a fixed order, so results are deterministic and agree with the
// sequential FP64 oracle to rounding.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mcx_device.cuh"
#include "mcx_flathist.cuh"
#include "mcx_internal.h"

using namespace mcx;

namespace {

constexpr int kTauBlock = 512;
constexpr int kTauGroups = kTauBlock / 32;

__device__ __forceinline__ double trace_value(const TraceSrc& s, long long t) {
    if (s.type == TRACE_F64) return static_cast<const double*>(s.base)[t * s.stride];
    const long long* p = static_cast<const long long*>(s.base) + t * s.stride;
    double x = 0.0;
    for (int k = 0; k < s.ncols; ++k) x = x + s.coef[k] * (double)p[k];
    return x;
}

// Deterministic block sum (fixed shuffle tree, then the warps in order), broadcast.
__device__ double tau_block_sum(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        red[32] = t;
    }
    __syncthreads();
    return red[32];
}

__global__ void __launch_bounds__(kTauBlock) k_tau_int(const TraceSrc* __restrict__ srcs, double* work,
                                                       const long long* __restrict__ work_off, double c, double* taus) {
    __shared__ double red[33];
    __shared__ double s_part[kTauGroups][32];
    __shared__ int s_done;
    const TraceSrc s = srcs[blockIdx.x];
    if (s.skip) {
        if (threadIdx.x == 0) taus[blockIdx.x] = __longlong_as_double(0x7FF8000000000000ll);
        return;
    }
    double* ce = work + work_off[blockIdx.x];
    const long long n = s.n;
    double part = 0.0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const double x = trace_value(s, i);
        ce[i] = x;
        part += x;
    }
    const double mu = tau_block_sum(part, red) / (double)n;
    part = 0.0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {  // the same elements as above
        const double v = ce[i] - mu;
        ce[i] = v;
        part += v * v;
    }
    const double c0 = tau_block_sum(part, red) / (double)n;  // also orders the writes of ce
    double tau = 0.5;
    if (c0 > 0) {
        if (threadIdx.x == 0) s_done = 0;
        __syncthreads();
        const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
        for (long long lag0 = 1; lag0 <= s.cap; lag0 += 32) {
            const long long lag = lag0 + lane;
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
            if (lag <= s.cap) {
                const long long m = n - lag;
                long long i = grp;
                for (; i + 3 * kTauGroups < m; i += 4 * kTauGroups) {
                    a0 = fma(ce[i], ce[i + lag], a0);
                    a1 = fma(ce[i + kTauGroups], ce[i + kTauGroups + lag], a1);
                    a2 = fma(ce[i + 2 * kTauGroups], ce[i + 2 * kTauGroups + lag], a2);
                    a3 = fma(ce[i + 3 * kTauGroups], ce[i + 3 * kTauGroups + lag], a3);
                }
                for (; i < m; i += kTauGroups) a0 = fma(ce[i], ce[i + lag], a0);
            }
            s_part[grp][lane] = (a0 + a1) + (a2 + a3);
            __syncthreads();
            if (threadIdx.x < 32) {
                double cov = 0.0;
                for (int g = 0; g < kTauGroups; ++g) cov += s_part[g][threadIdx.x];
                s_part[0][threadIdx.x] = (cov / (double)(n - lag)) / c0;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int l = 0; l < 32 && lag0 + l <= s.cap; ++l) {
                    const double C = s_part[0][l];
                    if (C <= 0) {
                        s_done = 1;
                        break;
                    }
                    const double next = tau + C;
                    if ((double)(lag0 + l) > c * next) {
                        s_done = 1;
                        break;
                    }
                    tau = next;
                }
            }
            __syncthreads();
            if (s_done) break;
        }
    }
    if (threadIdx.x == 0) taus[blockIdx.x] = tau > 0.5 ? tau : 0.5;
}

// ---------------------------------------------------------------- reweighting --
// Canonical moments from a log density of states (distribution_from_logdos,
// src/infrastructure/utils.jl:95-105): for each beta, over the bins whose log weight
// w_b = ln g_b - beta E_b is finite, the log-sum-exp state (m, sum exp(w - m) (1, E, E^2)).
// A thread folds its bins in order (rescaling the sums when the maximum grows), a block
// merges its threads in a fixed tree, and one thread per beta merges the blocks in order,
// so results are deterministic; exp and log are mcx_exp / mcx_log.
constexpr int kRwBlock = 256;

struct Lse {
    double m, s0, s1, s2;
};

__device__ __forceinline__ void lse_add(Lse& a, double w, double E) {
    if (w > a.m) {
        const double f = mcx_exp(a.m - w);  // 0 while the state is empty (m = -inf)
        a.s0 = a.s0 * f;
        a.s1 = a.s1 * f;
        a.s2 = a.s2 * f;
        a.m = w;
    }
    const double e = mcx_exp(w - a.m);
    a.s0 = a.s0 + e;
    a.s1 = a.s1 + e * E;
    a.s2 = a.s2 + (e * E) * E;
}

__device__ __forceinline__ Lse lse_merge(Lse a, Lse b) {
    if (b.m > a.m) {
        const Lse t = a;
        a = b;
        b = t;
    }
    if (b.s0 == 0.0) return a;  // b is empty
    const double f = mcx_exp(b.m - a.m);
    a.s0 = a.s0 + b.s0 * f;
    a.s1 = a.s1 + b.s1 * f;
    a.s2 = a.s2 + b.s2 * f;
    return a;
}

__device__ __forceinline__ Lse lse_shfl(const Lse& a, int o) {
    return Lse{__shfl_down_sync(0xFFFFFFFFu, a.m, o), __shfl_down_sync(0xFFFFFFFFu, a.s0, o),
               __shfl_down_sync(0xFFFFFFFFu, a.s1, o), __shfl_down_sync(0xFFFFFFFFu, a.s2, o)};
}

// grid (blocks over the bins, betas): block x folds bins [x*per, (x+1)*per) at betas[y]
__global__ void __launch_bounds__(kRwBlock) k_reweight_partial(const double* __restrict__ lnw, long long nbins,
                                                               long long start, long long step,
                                                               const double* __restrict__ betas,
                                                               Lse* __restrict__ part) {
    __shared__ Lse red[kRwBlock / 32];
    const double beta = betas[blockIdx.y];
    const long long per = (nbins + gridDim.x - 1) / gridDim.x;
    const long long b0 = (long long)blockIdx.x * per;
    const long long b1 = b0 + per < nbins ? b0 + per : nbins;
    Lse a{-HUGE_VAL, 0.0, 0.0, 0.0};
    for (long long b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
        const double E = (double)(start + step * b);
        const double w = (-lnw[b]) - beta * E;  // ln g = -logweight
        if (isfinite(w)) lse_add(a, w, E);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a = lse_merge(a, lse_shfl(a, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        Lse t = red[0];
        for (int w = 1; w < kRwBlock / 32; ++w) t = lse_merge(t, red[w]);
        part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
    }
}

// one thread per beta: the blocks in order, then (log Z, <E>, <E^2>); log Z is NaN when
// no bin was finite
__global__ void k_reweight_finish(const Lse* __restrict__ part, int nblk, int nbeta, double* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nbeta) return;
    Lse t = part[(size_t)k * nblk];
    for (int x = 1; x < nblk; ++x) t = lse_merge(t, part[(size_t)k * nblk + x]);
    const bool any = t.s0 > 0.0;
    out[3 * k] = any ? t.m + mcx_log(t.s0) : __longlong_as_double(0x7FF8000000000000ll);
    out[3 * k + 1] = any ? t.s1 / t.s0 : 0.0;
    out[3 * k + 2] = any ? t.s2 / t.s0 : 0.0;
}

// the distribution at one beta: exp(w_b - log Z) on finite bins, 0 elsewhere
__global__ void k_reweight_dist(const double* __restrict__ lnw, long long nbins, long long start, long long step,
                                const double* __restrict__ beta, const double* __restrict__ logz,
                                double* __restrict__ dist) {
    const double bt = *beta, lz = *logz;
    for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < nbins;
         b += (long long)gridDim.x * blockDim.x) {
        const double w = (-lnw[b]) - bt * (double)(start + step * b);
        dist[b] = isfinite(w) ? mcx_exp(w - lz) : 0.0;
    }
}

}  // namespace

namespace mcx {

mcx_status launch_tau_int(mcx_ctx* ctx, const std::vector<TraceSrc>& srcs, const double* host_values,
                          size_t host_count, double c, double* taus) {
    const int nt = (int)srcs.size();
    if (nt == 0) return MCX_OK;
    // scratch: descriptors | work offsets | taus | host values | centred traces
    std::vector<long long> off(nt, 0);
    long long tot = 0;
    for (int k = 0; k < nt; ++k) {
        off[k] = tot;
        if (!srcs[k].skip) tot += srcs[k].n;
    }
    auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
    const size_t b_src = up16(sizeof(TraceSrc) * nt), b_off = up16(sizeof(long long) * nt),
                 b_tau = up16(sizeof(double) * nt), b_val = up16(sizeof(double) * host_count),
                 b_work = sizeof(double) * (size_t)(tot > 0 ? tot : 1);
    void* scratch = nullptr;
    MCX_CHECK(ctx_scratch(ctx, b_src + b_off + b_tau + b_val + b_work, &scratch));
    char* base = static_cast<char*>(scratch);
    TraceSrc* d_src = reinterpret_cast<TraceSrc*>(base);
    long long* d_off = reinterpret_cast<long long*>(base + b_src);
    double* d_tau = reinterpret_cast<double*>(base + b_src + b_off);
    double* d_val = reinterpret_cast<double*>(base + b_src + b_off + b_tau);
    double* d_work = reinterpret_cast<double*>(base + b_src + b_off + b_tau + b_val);
    std::vector<TraceSrc> s2(srcs);
    for (auto& s : s2)
        if (s.base == nullptr && s.type == TRACE_F64) s.base = d_val + s.host_offset;  // host traces
    cudaStream_t st = ctx->stream;
    MCX_CUDA(cudaMemcpyAsync(d_src, s2.data(), sizeof(TraceSrc) * nt, cudaMemcpyHostToDevice, st));
    MCX_CUDA(cudaMemcpyAsync(d_off, off.data(), sizeof(long long) * nt, cudaMemcpyHostToDevice, st));
    if (host_count)
        MCX_CUDA(cudaMemcpyAsync(d_val, host_values, sizeof(double) * host_count, cudaMemcpyHostToDevice, st));
    k_tau_int<<<nt, kTauBlock, 0, st>>>(d_src, d_work, d_off, c, d_tau);
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    MCX_CUDA(cudaMemcpyAsync(taus, d_tau, sizeof(double) * nt, cudaMemcpyDeviceToHost, st));
    MCX_CUDA(cudaStreamSynchronize(st));  // the host vectors above outlive the copies
    return MCX_OK;
}

// The lag window of a trace of n samples under the batch rules of
// integrated_autocorrelation_times (autocorrelations.jl:76-102): fewer than min_points
// samples or no positive window -> skipped (NaN).
void tau_window(TraceSrc& s, long long n, long long min_points, long long max_lag) {
    s.n = n;
    s.cap = max_lag > 0 ? std::min(max_lag, n / 2) : n / 2;
    s.skip = (n < min_points || n < 2 || s.cap < 1) ? 1 : 0;
}

}  // namespace mcx

extern "C" {

MCX_API mcx_status mcx_tau_int(mcx_ctx* ctx, const double* values, const int64_t* offsets, int32_t ntraces,
                               int64_t min_points, int64_t max_lag, double c, double* taus) {
    if (!ctx || !offsets || !taus || (ntraces > 0 && !values)) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (ntraces < 0) return fail(MCX_ERR_INVALID_ARG, "ntraces < 0");
    if (!(c > 0)) return fail(MCX_ERR_INVALID_ARG, "c must be positive");
    if (min_points < 2) return fail(MCX_ERR_INVALID_ARG, "min_points must be >= 2");
    if (offsets[0] < 0) return fail(MCX_ERR_INVALID_ARG, "offsets[0] < 0");
    std::vector<TraceSrc> srcs(ntraces);
    for (int k = 0; k < ntraces; ++k) {
        const long long n = offsets[k + 1] - offsets[k];
        if (n < 0) return fail(MCX_ERR_INVALID_ARG, "offsets decrease at trace %d", k);
        TraceSrc& s = srcs[k];
        s = TraceSrc{};
        s.type = TRACE_F64;
        s.stride = 1;
        s.base = nullptr;
        s.host_offset = offsets[k] - offsets[0];
        tau_window(s, n, min_points, max_lag);
    }
    const size_t count = ntraces > 0 ? (size_t)(offsets[ntraces] - offsets[0]) : 0;
    return launch_tau_int(ctx, srcs, values + (ntraces > 0 ? offsets[0] : 0), count, c, taus);
}

MCX_API mcx_status mcx_lattice_tau_int(mcx_lattice* lat, int quantity, int64_t max_lag, double c, double* tau) {
    if (!lat || !tau) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (quantity != 0 && quantity != 1) return fail(MCX_ERR_INVALID_ARG, "quantity must be 0 (energy) or 1 (magnetization)");
    if (!(c > 0)) return fail(MCX_ERR_INVALID_ARG, "c must be positive");
    const long long n = lat->series_len;
    if (n < 2) return fail(MCX_ERR_INVALID_ARG, "the last sweep call recorded %lld sweeps (at least 2 needed)", n);
    if (max_lag > n / 2) return fail(MCX_ERR_INVALID_ARG, "max_lag must satisfy 1 <= max_lag <= floor(n/2)");
    std::vector<TraceSrc> srcs(1);
    TraceSrc& s = srcs[0];
    s = TraceSrc{};
    s.base = lat->d_series;
    s.type = TRACE_I64;
    s.stride = 3;
    s.ncols = 3;
    if (quantity == 0) {  // -J pair - h spin (+ D spin2)
        s.coef[0] = -lat->J;
        s.coef[1] = -lat->h;
        s.coef[2] = lat->model == MCX_BLUME_CAPEL ? lat->D : 0.0;
    } else {
        s.coef[1] = 1.0;
    }
    tau_window(s, n, 2, max_lag);
    return launch_tau_int(lat->ctx, srcs, nullptr, 0, c, tau);
}

MCX_API mcx_status mcx_flathist_reweight(mcx_flathist* fh, const double* betas, int32_t nbeta, double* logz,
                                         double* mean_e, double* mean_e2, double* dist, int64_t dist_len) {
    if (!fh || !betas || !logz || !mean_e || !mean_e2) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (nbeta < 1 || nbeta > 65535) return fail(MCX_ERR_INVALID_ARG, "nbeta must be in 1..65535");
    if (dist && dist_len != fh->nbins)
        return fail(MCX_ERR_INVALID_ARG, "the distribution needs %lld entries", (long long)fh->nbins);
    for (int k = 0; k < nbeta; ++k)
        if (!std::isfinite(betas[k])) return fail(MCX_ERR_INVALID_ARG, "beta %d must be finite", k);
    mcx_ctx* ctx = fh->ctx;
    const long long nbins = fh->nbins;
    // about 8 blocks per SM over all betas, at least 4 * kRwBlock bins per block
    const long long by_bins = (nbins + 4 * kRwBlock - 1) / (4 * kRwBlock);
    const long long by_grid = std::max<long long>(1, 8LL * std::max(ctx->num_sms, 1) / nbeta);
    const int nblk = (int)std::max<long long>(1, std::min(by_bins, by_grid));
    auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
    const size_t b_beta = up16(sizeof(double) * nbeta), b_out = up16(sizeof(double) * 3 * nbeta);
    const size_t b_part = up16(sizeof(Lse) * (size_t)nbeta * nblk);
    const size_t b_dist = dist ? sizeof(double) * (size_t)nbins : 0;
    // scratch: betas | (log Z, <E>, <E^2>) per beta | block partials | the distribution
    void* scratch = nullptr;
    MCX_CHECK(ctx_scratch(ctx, b_beta + b_out + b_part + b_dist, &scratch));
    char* base = static_cast<char*>(scratch);
    double* d_beta = reinterpret_cast<double*>(base);
    double* d_out = reinterpret_cast<double*>(base + b_beta);
    Lse* d_part = reinterpret_cast<Lse*>(base + b_beta + b_out);
    double* d_dist = reinterpret_cast<double*>(base + b_beta + b_out + b_part);
    cudaStream_t st = ctx->stream;
    MCX_CUDA(cudaMemcpyAsync(d_beta, betas, sizeof(double) * nbeta, cudaMemcpyHostToDevice, st));
    k_reweight_partial<<<dim3((unsigned)nblk, (unsigned)nbeta), kRwBlock, 0, st>>>(fh->d_lnw, nbins, fh->start,
                                                                                  fh->step, d_beta, d_part);
    k_reweight_finish<<<(nbeta + 127) / 128, 128, 0, st>>>(d_part, nblk, nbeta, d_out);
    count_launch(ctx, 2);
    if (dist) {
        const unsigned grid = (unsigned)std::min<long long>((nbins + 255) / 256, 8LL * std::max(ctx->num_sms, 1));
        k_reweight_dist<<<grid, 256, 0, st>>>(fh->d_lnw, nbins, fh->start, fh->step, d_beta, d_out, d_dist);
        count_launch(ctx);
    }
    MCX_CUDA(cudaGetLastError());
    std::vector<double> out(3 * (size_t)nbeta);
    MCX_CUDA(cudaMemcpyAsync(out.data(), d_out, sizeof(double) * 3 * nbeta, cudaMemcpyDeviceToHost, st));
    if (dist) MCX_CUDA(cudaMemcpyAsync(dist, d_dist, b_dist, cudaMemcpyDeviceToHost, st));
    MCX_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < nbeta; ++k) {
        if (std::isnan(out[3 * k])) return fail(MCX_ERR_INVALID_ARG, "the log density of states has no finite entry");
        logz[k] = out[3 * k];
        mean_e[k] = out[3 * k + 1];
        mean_e2[k] = out[3 * k + 2];
    }
    return MCX_OK;
}

}  // extern "C"

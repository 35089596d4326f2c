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

}  // extern "C"

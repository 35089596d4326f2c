// mcx_core.cu -- context, lattice storage, layout conversion, observables and the
// host-side acceptance tables of libmcx_cuda.
//
// Device layout (INT8): the lattice is split by colour (x+y+z)&1 into two arrays of
// rows r = y + Ly*z, each row holding W = Lx/2 bytes; entry k of colour c in row r is
// the site x = 2k + ((y+z+c)&1).  A checkerboard half-sweep then reads one whole
// array (the other colour), reads and writes the other (its own colour) with dense
// 128-bit accesses.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>

#include "mcx_device.cuh"
#include "mcx_internal.h"

namespace mcx {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

mcx_status fail(mcx_status st, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return st;
}

mcx_status cuda_fail(cudaError_t e, const char* what) {
    set_error("%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? MCX_ERR_OOM : MCX_ERR_CUDA;
}

void ctx_release(mcx_ctx* ctx) {
    if (ctx->refs.fetch_sub(1) != 1) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->capture_stream) cudaStreamDestroy(ctx->capture_stream);
    if (ctx->d_scratch) cudaFree(ctx->d_scratch);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

mcx_status ctx_scratch(mcx_ctx* ctx, size_t bytes, void** out) {
    if (bytes > ctx->scratch_bytes) {
        size_t cap = ctx->scratch_bytes ? ctx->scratch_bytes : 4096;
        while (cap < bytes) cap *= 2;
        if (ctx->budget && ctx->used - ctx->scratch_bytes + cap > ctx->budget)
            return fail(MCX_ERR_BUDGET, "HBM budget exceeded by %zu scratch bytes", cap);
        MCX_CUDA(cudaStreamSynchronize(ctx->stream));  // the old scratch may still be read
        if (ctx->d_scratch) cudaFree(ctx->d_scratch);
        ctx->used -= ctx->scratch_bytes;
        ctx->d_scratch = nullptr;
        ctx->scratch_bytes = 0;
        MCX_CUDA(cudaMalloc(&ctx->d_scratch, cap));
        ctx->scratch_bytes = cap;
        ctx->used += cap;
    }
    *out = ctx->d_scratch;
    return MCX_OK;
}

mcx_status dev_alloc(mcx_ctx* ctx, void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return MCX_OK;
    if (ctx->budget && ctx->used + bytes > ctx->budget)
        return fail(MCX_ERR_BUDGET, "allocation of %zu bytes exceeds the HBM budget (%llu of %llu used)",
                    bytes, (unsigned long long)ctx->used, (unsigned long long)ctx->budget);
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    ctx->used += bytes;
    return MCX_OK;
}

void dev_free(mcx_ctx* ctx, void* p, size_t bytes) {
    if (!p) return;
    cudaFree(p);
    ctx->used -= bytes;
}

// ------------------------------------------------------------------ tables --
// logistic, src/infrastructure/utils.jl:82-88
static double logistic(double x) {
    if (x >= 0) return 1.0 / (1.0 + std::exp(-x));
    double ex = std::exp(x);
    return ex / (1.0 + ex);
}

// floor(p * 2^32); 2^32 stands for "always"
static uint64_t threshold(double p) {
    if (!(p > 0.0)) return 0;
    if (p >= 1.0) return 1ull << 32;
    double v = std::floor(p * 4294967296.0);
    return v >= 4294967296.0 ? (1ull << 32) : (uint64_t)v;
}

// accept iff lr > 0 || U < exp(lr), lr = -beta*dE
// (src/algorithms/metropolis.jl:14-17, importance_sampling.jl:80-85, boltzmann.jl:28)
static uint64_t metropolis(double beta, double dE) {
    double lr = (-beta) * dE;
    if (lr >= 0.0) return 1ull << 32;
    return threshold(std::exp(lr));
}

// accept iff U < logistic(lr)  (src/algorithms/metropolis.jl:121-127)
static uint64_t glauber(double beta, double dE) { return threshold(logistic((-beta) * dE)); }

// Ising: entry a + (2d+1)*up, a = aligned neighbours; flip iff (u ^ m) < thr with
// m = ~0 for heat-bath entries of an up spin, else 0.
mcx_status build_ising_table(int dim, mcx_algorithm alg, double beta, double J, double h,
                             Table* t) {
    const int z = 2 * dim;
    t->n = 2 * (z + 1);
    for (int up = 0; up < 2; ++up)
        for (int a = 0; a <= z; ++a) {
            const double s = up ? 1.0 : -1.0;
            const double lpi = (double)(2 * a - z);
            const double dpair = ((-2.0) * J) * lpi;     // flip_changes, SpinSystems/src/ising.jl:484-489
            const double dE = (-dpair) - (h * (-2.0 * s));  // delta_energy, ising.jl:198
            uint64_t v;
            if (alg == MCX_METROPOLIS) v = metropolis(beta, dE);
            else if (alg == MCX_GLAUBER) v = glauber(beta, dE);
            else if (alg == MCX_HEATBATH) {
                // ising.jl:43-58: p_plus = logistic(beta*s_old*dE); s_new = U<p_plus ? +1 : -1
                const uint64_t tp = threshold(logistic((beta * s) * dE));
                v = up ? (1ull << 32) - tp : tp;
            } else
                return fail(MCX_ERR_INVALID_ARG, "unknown algorithm %d", (int)alg);
            t->thr[a + (z + 1) * up] = v;
        }
    return MCX_OK;
}

// _propose_state, SpinSystems/src/blume_capel.jl:21-30
static int bc_propose(int s_old, int b) {
    if (s_old == -1) return b ? 0 : 1;
    if (s_old == 0) return b ? -1 : 1;
    return b ? -1 : 0;
}

// Blume-Capel: Metropolis/Glauber entry (s_old+1)*2*nc + b*nc + (c+z), nc = 2z+1;
// heat bath: per neighbour sum c the cumulative thresholds (T1, T12) at 2(c+z), 2(c+z)+1.
mcx_status build_bc_table(int dim, mcx_algorithm alg, double beta, double J, double D,
                          double h, Table* t) {
    const int z = 2 * dim, nc = 2 * z + 1;
    if (alg == MCX_HEATBATH) {
        t->n = 2 * nc;
        for (int c = -z; c <= z; ++c) {
            // blume_capel.jl:61-85
            const double coupling = J * (double)c;
            const double e1 = (coupling - (h * -1.0)) + D;
            const double e3 = ((-coupling) - (h * 1.0)) + D;
            const double w1 = std::exp((-beta) * e1);
            const double w2 = std::exp((-beta) * 0.0);
            const double w3 = std::exp((-beta) * e3);
            const double zz = (w1 + w2) + w3;
            t->thr[2 * (c + z)] = threshold(w1 / zz);
            t->thr[2 * (c + z) + 1] = threshold((w1 + w2) / zz);
        }
        return MCX_OK;
    }
    if (alg != MCX_METROPOLIS && alg != MCX_GLAUBER)
        return fail(MCX_ERR_INVALID_ARG, "unknown algorithm %d", (int)alg);
    t->n = 3 * 2 * nc;
    for (int so = -1; so <= 1; ++so)
        for (int b = 0; b < 2; ++b)
            for (int c = -z; c <= z; ++c) {
                const int sn = bc_propose(so, b);
                const double ds = (double)(sn - so), ds2 = (double)(sn * sn - so * so);
                const double dpair = ds * (J * (double)c);          // blume_capel.jl:235-241
                const double dE = ((-dpair) - (h * ds)) + (D * ds2);  // blume_capel.jl:247-248
                t->thr[(so + 1) * 2 * nc + b * nc + (c + z)] =
                    alg == MCX_METROPOLIS ? metropolis(beta, dE) : glauber(beta, dE);
            }
    return MCX_OK;
}

// ---------------------------------------------------------------- kernels --
struct Geo {
    int W, Ly, Lz, Lx;
    long long N;
};

__device__ __forceinline__ void site_of(const Geo& g, long long i, int& x, int& y, int& z) {
    x = (int)(i % g.Lx);
    long long rr = i / g.Lx;
    y = (int)(rr % g.Ly);
    z = (int)(rr / g.Ly);
}

__global__ void k_scatter(const int8_t* __restrict__ lin, int8_t* __restrict__ c0,
                          int8_t* __restrict__ c1, Geo g) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < g.N;
         i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        site_of(g, i, x, y, z);
        const long long e = (long long)(y + g.Ly * z) * g.W + (x >> 1);
        ((x + y + z) & 1 ? c1 : c0)[e] = lin[i];
    }
}

__global__ void k_gather(int8_t* __restrict__ lin, const int8_t* __restrict__ c0,
                         const int8_t* __restrict__ c1, Geo g) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < g.N;
         i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        site_of(g, i, x, y, z);
        const long long e = (long long)(y + g.Ly * z) * g.W + (x >> 1);
        lin[i] = ((x + y + z) & 1 ? c1 : c0)[e];
    }
}

// Number of bytes that are not spin states of the model (Ising {-1,+1}, BC {-1,0,+1}).
__global__ void k_validate(const int8_t* __restrict__ lin, long long n, int bc, unsigned long long* bad) {
    unsigned long long cnt = 0;
    const long long n16 = n / 16;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n16; q += stride) {
        const uint4 v = reinterpret_cast<const uint4*>(lin)[q];
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            uint32_t ok = __vcmpeq4(w[i], 0x01010101u) | __vcmpeq4(w[i], 0xFFFFFFFFu);
            if (bc) ok |= __vcmpeq4(w[i], 0u);
            cnt += __popc(~ok) >> 3;
        }
    }
    for (long long i = n16 * 16 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        const int v = lin[i];
        cnt += !(v == 1 || v == -1 || (bc && v == 0));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xFFFFFFFFu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(bad, cnt);
}

// Layout conversion 16 linear sites at a time (rows a multiple of 16 long): the even
// bytes of a chunk belong to one colour, the odd bytes to the other, and land as 8
// consecutive bytes in each colour array.
__global__ void k_scatter16(const uint4* __restrict__ lin, int8_t* __restrict__ c0, int8_t* __restrict__ c1, Geo g) {
    const long long cpr = g.Lx / 16, nq = g.N / 16;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nq;
         q += (long long)gridDim.x * blockDim.x) {
        const long long r = q / cpr;
        const int x0 = (int)(q - r * cpr) * 16;
        const int y = (int)(r % g.Ly), z = (int)(r / g.Ly);
        const int p0 = (y + z) & 1;  // colour of the even bytes
        const uint4 v = lin[q];
        const uint2 ev = make_uint2(__byte_perm(v.x, v.y, 0x6420), __byte_perm(v.z, v.w, 0x6420));
        const uint2 od = make_uint2(__byte_perm(v.x, v.y, 0x7531), __byte_perm(v.z, v.w, 0x7531));
        const long long e = r * g.W + (x0 >> 1);
        *reinterpret_cast<uint2*>((p0 ? c1 : c0) + e) = ev;
        *reinterpret_cast<uint2*>((p0 ? c0 : c1) + e) = od;
    }
}

__global__ void k_gather16(uint4* __restrict__ lin, const int8_t* __restrict__ c0, const int8_t* __restrict__ c1,
                           Geo g) {
    const long long cpr = g.Lx / 16, nq = g.N / 16;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nq;
         q += (long long)gridDim.x * blockDim.x) {
        const long long r = q / cpr;
        const int x0 = (int)(q - r * cpr) * 16;
        const int y = (int)(r % g.Ly), z = (int)(r / g.Ly);
        const int p0 = (y + z) & 1;
        const long long e = r * g.W + (x0 >> 1);
        const uint2 ev = *reinterpret_cast<const uint2*>((p0 ? c1 : c0) + e);
        const uint2 od = *reinterpret_cast<const uint2*>((p0 ? c0 : c1) + e);
        lin[q] = make_uint4(__byte_perm(ev.x, od.x, 0x5140), __byte_perm(ev.x, od.x, 0x7362),
                            __byte_perm(ev.y, od.y, 0x5140), __byte_perm(ev.y, od.y, 0x7362));
    }
}

// init!(sys, :random): Ising s = top bit ? +1 : -1; Blume-Capel s = floor(3u/2^32) - 1.
__global__ void k_init_random(int8_t* __restrict__ c0, int8_t* __restrict__ c1, Geo g,
                              uint32_t k0, uint32_t k1, uint32_t stream, int bc) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < g.N;
         i += (long long)gridDim.x * blockDim.x) {
        int x, y, z;
        site_of(g, i, x, y, z);
        const int c = (x + y + z) & 1;
        const uint4 w = philox10(make_uint4((uint32_t)(i >> 3), 0u, ctr_word2(0ull, c, P_INIT), stream), k0, k1);
        const uint32_t r = pick4(w, (int)((i >> 1) & 3));
        const int8_t s = bc ? (int8_t)((int)(((unsigned long long)r * 3ull) >> 32) - 1)
                            : (int8_t)((r & 0x80000000u) ? 1 : -1);
        const long long e = (long long)(y + g.Ly * z) * g.W + (x >> 1);
        (c ? c1 : c0)[e] = s;
    }
}

// Full recompute of (pair_sum, spin_sum, spin2_sum).  Every bond joins the two
// colours, so pair_sum = sum over colour-0 sites of s_i * (sum of its neighbours).
// Grid: x over the entries of a row, y over rows.
__global__ void k_observables(const int8_t* __restrict__ c0, const int8_t* __restrict__ c1,
                              Geo g, int dim, unsigned long long* state) {
    long long P = 0, M = 0, Q = 0;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int rows = g.Ly * g.Lz;
    if (k < g.W) {
        const int km = k == 0 ? g.W - 1 : k - 1, kp = k == g.W - 1 ? 0 : k + 1;
        for (int r = blockIdx.y; r < rows; r += gridDim.y) {
            const int y = r % g.Ly, z = r / g.Ly;
            const int p = (y + z) & 1;  // colour-0 parity of this row
            const long long rowb = (long long)r * g.W;
            const long long e = rowb + k;
            const int s = c0[e];
            int S = c1[e] + c1[rowb + (p ? kp : km)];
            const int yp = y + 1 == g.Ly ? 0 : y + 1, ym = y == 0 ? g.Ly - 1 : y - 1;
            S += c1[(long long)(yp + g.Ly * z) * g.W + k] + c1[(long long)(ym + g.Ly * z) * g.W + k];
            if (dim == 3) {
                const int zp = z + 1 == g.Lz ? 0 : z + 1, zm = z == 0 ? g.Lz - 1 : z - 1;
                S += c1[(long long)(y + g.Ly * zp) * g.W + k] + c1[(long long)(y + g.Ly * zm) * g.W + k];
            }
            const int s1 = c1[e];
            P += s * S;
            M += s + s1;
            Q += s * s + s1 * s1;
        }
    }
    long long v[3] = {P, M, Q};
    unsigned long long* const dst[3] = {state, state + 1, state + 2};
    block_add_atomic<3>(v, dst);
}

// series[s][j] = state[j] + sum_{s' <= s} delta[s'][j]; state := last row.
__global__ void k_prefix_series(long long* series, long long* state, long long n) {
    const int j = threadIdx.x;
    if (j >= 3) return;
    long long acc = state[j];
    for (long long s = 0; s < n; ++s) {
        acc += series[3 * s + j];
        series[3 * s + j] = acc;
    }
    state[j] = acc;
}

static int grid_for(const mcx_ctx* ctx, long long work, int block, int per_sm = 8) {
    long long g = (work + block - 1) / block;
    long long cap = (long long)ctx->num_sms * per_sm;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

static Geo geo_of(const mcx_lattice* lat) {
    Geo g;
    g.W = (int)lat->W;
    g.Ly = (int)lat->L[1];
    g.Lz = (int)lat->L[2];
    g.Lx = (int)lat->L[0];
    g.N = lat->N;
    return g;
}

mcx_status ensure_series(mcx_lattice* lat, int64_t nsweeps) {
    if (nsweeps <= lat->series_cap) return MCX_OK;
    int64_t cap = lat->series_cap ? lat->series_cap : 64;
    while (cap < nsweeps) cap *= 2;
    void* p = nullptr;
    MCX_CHECK(dev_alloc(lat->ctx, &p, (size_t)cap * 3 * sizeof(int64_t)));
    clear_graphs(lat);  // captured sweep sequences point at the old buffer
    dev_free(lat->ctx, lat->d_series, (size_t)lat->series_cap * 3 * sizeof(int64_t));
    lat->device_bytes += (cap - lat->series_cap) * 3 * (int64_t)sizeof(int64_t);
    lat->d_series = (int64_t*)p;
    lat->series_cap = cap;
    return MCX_OK;
}

mcx_status launch_prefix(mcx_lattice* lat, int64_t nsweeps, cudaStream_t stream) {
    k_prefix_series<<<1, 32, 0, stream>>>((long long*)lat->d_series, (long long*)lat->d_state, nsweeps);
    count_launch(lat->ctx);
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

mcx_status finish_series(mcx_lattice* lat, int64_t nsweeps) {
    MCX_CHECK(launch_prefix(lat, nsweeps, lat->ctx->stream));
    lat->series_len = nsweeps;
    return MCX_OK;
}

void clear_graphs(mcx_lattice* lat) {
    for (auto& g : lat->graphs) cudaGraphExecDestroy(g.exec);
    lat->graphs.clear();
}

mcx_status msc_pack(mcx_lattice* lat);    // mcx_msc.cu
mcx_status msc_unpack(mcx_lattice* lat);  // mcx_msc.cu

mcx_status recompute_state(mcx_lattice* lat) {
    mcx_ctx* ctx = lat->ctx;
    if (lat->layout == MCX_LAYOUT_MSC64) MCX_CHECK(msc_unpack(lat));
    MCX_CUDA(cudaMemsetAsync(lat->d_state, 0, 3 * sizeof(int64_t), ctx->stream));
    const Geo g = geo_of(lat);
    const int bx = (int)((lat->W + 255) / 256);
    int by = (int)std::min<int64_t>(lat->rows, 65535);
    by = std::max(1, std::min(by, (ctx->num_sms * 16 + bx - 1) / bx));
    k_observables<<<dim3(bx, by), 256, 0, ctx->stream>>>(lat->d_col[0], lat->d_col[1], g, lat->dim,
                                                          (unsigned long long*)lat->d_state);
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

}  // namespace mcx

using namespace mcx;

// ------------------------------------------------------------------- C ABI --
extern "C" {

MCX_API int mcx_version(void) { return 1; }

MCX_API const char* mcx_status_string(mcx_status s) {
    switch (s) {
        case MCX_OK: return "ok";
        case MCX_ERR_INVALID_ARG: return "invalid argument";
        case MCX_ERR_OUT_OF_RANGE: return "energy out of the histogram range";
        case MCX_ERR_OOM: return "out of device memory";
        case MCX_ERR_BUDGET: return "HBM budget exceeded";
        case MCX_ERR_TIMEOUT: return "device-side wait timed out";
        case MCX_ERR_CUDA: return "CUDA error";
        case MCX_ERR_NOT_READY: return "not ready";
        case MCX_ERR_NOT_FOUND: return "not found";
    }
    return "unknown status";
}

MCX_API const char* mcx_last_error_string(void) { return g_err; }

MCX_API mcx_status mcx_ctx_create(const mcx_config* cfg, mcx_ctx** out) {
    if (!out) return fail(MCX_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    mcx_config c{};
    if (cfg) c = *cfg;
    int ndev = 0;
    MCX_CUDA(cudaGetDeviceCount(&ndev));
    if (c.device < 0 || c.device >= ndev) return fail(MCX_ERR_INVALID_ARG, "device %d of %d", c.device, ndev);
    MCX_CUDA(cudaSetDevice(c.device));
    mcx_ctx* ctx = new mcx_ctx();
    ctx->device = c.device;
    ctx->budget = c.hbm_budget;
    cudaError_t e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, c.device);
    if (e != cudaSuccess) {
        delete ctx;
        return cuda_fail(e, "cudaDeviceGetAttribute");
    }
    if (c.stream) {
        ctx->stream = (cudaStream_t)c.stream;
    } else {
        e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete ctx;
            return cuda_fail(e, "cudaStreamCreate");
        }
        ctx->own_stream = true;
    }
    *out = ctx;
    return MCX_OK;
}

MCX_API mcx_status mcx_ctx_destroy(mcx_ctx* ctx) {
    if (!ctx) return MCX_OK;
    cudaStreamSynchronize(ctx->stream);
    ctx_release(ctx);
    return MCX_OK;
}

MCX_API mcx_status mcx_sync(mcx_ctx* ctx) {
    if (!ctx) return fail(MCX_ERR_INVALID_ARG, "ctx is NULL");
    MCX_CUDA(cudaStreamSynchronize(ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_ctx_stream(mcx_ctx* ctx, void** stream) {
    if (!ctx || !stream) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    *stream = (void*)ctx->stream;
    return MCX_OK;
}

MCX_API mcx_status mcx_ctx_memory(mcx_ctx* ctx, uint64_t* used, uint64_t* budget) {
    if (!ctx) return fail(MCX_ERR_INVALID_ARG, "ctx is NULL");
    if (used) *used = ctx->used;
    if (budget) *budget = ctx->budget;
    return MCX_OK;
}

MCX_API mcx_status mcx_ctx_launches(mcx_ctx* ctx, uint64_t* launches) {
    if (!ctx || !launches) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    *launches = ctx->launches;
    return MCX_OK;
}

MCX_API mcx_status mcx_lattice_create(mcx_ctx* ctx, mcx_model model, int dim, const int32_t* L,
                                      mcx_layout layout, double J, double D, double h,
                                      mcx_lattice** out) {
    if (!ctx || !L || !out) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (dim != 2 && dim != 3) return fail(MCX_ERR_INVALID_ARG, "dim must be 2 or 3 (got %d)", dim);
    if (model != MCX_ISING && model != MCX_BLUME_CAPEL) return fail(MCX_ERR_INVALID_ARG, "unknown model");
    if (layout != MCX_LAYOUT_INT8 && layout != MCX_LAYOUT_MSC64) return fail(MCX_ERR_INVALID_ARG, "unknown layout");
    if (!std::isfinite(J) || !std::isfinite(D) || !std::isfinite(h))
        return fail(MCX_ERR_INVALID_ARG, "J, D and h must be finite");
    int64_t N = 1;
    for (int d = 0; d < dim; ++d) {
        if (L[d] < 4 || (L[d] & 1))
            return fail(MCX_ERR_INVALID_ARG, "side %d is %d: checkerboard sweeps need even sides >= 4", d, L[d]);
        N *= L[d];
    }
    if (N > (1ll << 34)) return fail(MCX_ERR_INVALID_ARG, "lattice too large");
    if (layout == MCX_LAYOUT_MSC64) {
        if (model != MCX_ISING) return fail(MCX_ERR_INVALID_ARG, "MSC64 layout holds Ising spins only");
        if (L[0] % 128) return fail(MCX_ERR_INVALID_ARG, "MSC64 layout needs Lx a multiple of 128");
    }
    mcx_lattice* lat = new mcx_lattice();
    lat->ctx = ctx;
    lat->hold.set(ctx);
    lat->model = model;
    lat->layout = layout;
    lat->dim = dim;
    lat->L[0] = L[0];
    lat->L[1] = L[1];
    lat->L[2] = dim == 3 ? L[2] : 1;
    lat->J = J;
    lat->D = D;
    lat->h = h;
    lat->N = N;
    lat->W = L[0] / 2;
    lat->rows = lat->L[1] * lat->L[2];
    const size_t half = (size_t)(N / 2);
    mcx_status st = MCX_OK;
    void* p = nullptr;
    auto grab = [&](void** dst, size_t bytes) {
        if (st != MCX_OK) return;
        st = dev_alloc(ctx, dst, bytes);
        if (st == MCX_OK) lat->device_bytes += (int64_t)bytes;
    };
    grab((void**)&lat->d_col[0], half);
    grab((void**)&lat->d_col[1], half);
    if (layout == MCX_LAYOUT_MSC64) {
        grab((void**)&lat->d_msc[0], half / 8);
        grab((void**)&lat->d_msc[1], half / 8);
    }
    grab((void**)&lat->d_lin, (size_t)N);
    grab((void**)&lat->d_state, 3 * sizeof(int64_t));
    grab(&p, sizeof(unsigned long long));
    lat->d_acc = (unsigned long long*)p;
    grab(&p, 4 * sizeof(unsigned long long));
    lat->d_sweep_base = (unsigned long long*)p;
    if (st == MCX_OK) st = ensure_series(lat, 64);
    if (st != MCX_OK) {
        mcx_lattice_destroy(lat);
        return st;
    }
    *out = lat;
    return mcx_init_uniform(lat, 1);
}

MCX_API mcx_status mcx_lattice_destroy(mcx_lattice* lat) {
    if (!lat) return MCX_OK;
    mcx_ctx* ctx = lat->ctx;
    cudaStreamSynchronize(ctx->stream);
    const size_t half = (size_t)(lat->N / 2);
    dev_free(ctx, lat->d_col[0], half);
    dev_free(ctx, lat->d_col[1], half);
    dev_free(ctx, lat->d_msc[0], half / 8);
    dev_free(ctx, lat->d_msc[1], half / 8);
    dev_free(ctx, lat->d_lin, (size_t)lat->N);
    dev_free(ctx, lat->d_state, 3 * sizeof(int64_t));
    dev_free(ctx, lat->d_acc, sizeof(unsigned long long));
    dev_free(ctx, lat->d_sweep_base, 4 * sizeof(unsigned long long));
    clear_graphs(lat);
    dev_free(ctx, lat->d_series, (size_t)lat->series_cap * 3 * sizeof(int64_t));
    delete lat;
    return MCX_OK;
}

MCX_API mcx_status mcx_lattice_info(const mcx_lattice* lat, int64_t* nsites, int64_t* device_bytes) {
    if (!lat) return fail(MCX_ERR_INVALID_ARG, "lattice is NULL");
    if (nsites) *nsites = lat->N;
    if (device_bytes) *device_bytes = lat->device_bytes;
    return MCX_OK;
}

MCX_API mcx_status mcx_set_spins(mcx_lattice* lat, const int8_t* host, size_t n) {
    if (!lat || !host) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if ((int64_t)n != lat->N) return fail(MCX_ERR_INVALID_ARG, "expected %lld spins, got %zu", (long long)lat->N, n);
    mcx_ctx* ctx = lat->ctx;
    MCX_CUDA(cudaMemcpyAsync(lat->d_lin, host, n, cudaMemcpyHostToDevice, ctx->stream));
    // validate on the device before the lattice is touched (the counter word is free here)
    unsigned long long bad = 0;
    MCX_CUDA(cudaMemsetAsync(lat->d_acc, 0, sizeof(unsigned long long), ctx->stream));
    k_validate<<<grid_for(ctx, lat->N / 16 + 1, 256), 256, 0, ctx->stream>>>(lat->d_lin, lat->N,
                                                                             lat->model == MCX_BLUME_CAPEL, lat->d_acc);
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    MCX_CUDA(cudaMemcpyAsync(&bad, lat->d_acc, sizeof(bad), cudaMemcpyDeviceToHost, ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (bad) return fail(MCX_ERR_INVALID_ARG, "%llu values are not spin states of this model", bad);
    const Geo g = geo_of(lat);
    if (lat->L[0] % 16 == 0)
        k_scatter16<<<grid_for(ctx, lat->N / 16, 256), 256, 0, ctx->stream>>>(
            reinterpret_cast<const uint4*>(lat->d_lin), lat->d_col[0], lat->d_col[1], g);
    else
        k_scatter<<<grid_for(ctx, lat->N, 256), 256, 0, ctx->stream>>>(lat->d_lin, lat->d_col[0], lat->d_col[1], g);
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    if (lat->layout == MCX_LAYOUT_MSC64) MCX_CHECK(msc_pack(lat));
    return recompute_state(lat);
}

MCX_API mcx_status mcx_get_spins(mcx_lattice* lat, int8_t* host, size_t n) {
    if (!lat || !host) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if ((int64_t)n != lat->N) return fail(MCX_ERR_INVALID_ARG, "expected %lld spins, got %zu", (long long)lat->N, n);
    mcx_ctx* ctx = lat->ctx;
    if (lat->layout == MCX_LAYOUT_MSC64) MCX_CHECK(msc_unpack(lat));
    const Geo g = geo_of(lat);
    if (lat->L[0] % 16 == 0)
        k_gather16<<<grid_for(ctx, lat->N / 16, 256), 256, 0, ctx->stream>>>(reinterpret_cast<uint4*>(lat->d_lin),
                                                                             lat->d_col[0], lat->d_col[1], g);
    else
        k_gather<<<grid_for(ctx, lat->N, 256), 256, 0, ctx->stream>>>(lat->d_lin, lat->d_col[0], lat->d_col[1], g);
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    MCX_CUDA(cudaMemcpyAsync(host, lat->d_lin, n, cudaMemcpyDeviceToHost, ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(ctx->stream));
    return MCX_OK;
}

MCX_API mcx_status mcx_init_random(mcx_lattice* lat, uint64_t seed, uint32_t stream) {
    if (!lat) return fail(MCX_ERR_INVALID_ARG, "lattice is NULL");
    mcx_ctx* ctx = lat->ctx;
    const Geo g = geo_of(lat);
    k_init_random<<<grid_for(ctx, lat->N, 256), 256, 0, ctx->stream>>>(
        lat->d_col[0], lat->d_col[1], g, (uint32_t)seed, (uint32_t)(seed >> 32), stream,
        lat->model == MCX_BLUME_CAPEL);
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    if (lat->layout == MCX_LAYOUT_MSC64) MCX_CHECK(msc_pack(lat));
    return recompute_state(lat);
}

MCX_API mcx_status mcx_init_uniform(mcx_lattice* lat, int8_t value) {
    if (!lat) return fail(MCX_ERR_INVALID_ARG, "lattice is NULL");
    const bool ok = lat->model == MCX_ISING ? (value == 1 || value == -1) : (value >= -1 && value <= 1);
    if (!ok) return fail(MCX_ERR_INVALID_ARG, "value %d is not a spin state of this model", (int)value);
    mcx_ctx* ctx = lat->ctx;
    MCX_CUDA(cudaMemsetAsync(lat->d_col[0], (unsigned char)value, (size_t)(lat->N / 2), ctx->stream));
    MCX_CUDA(cudaMemsetAsync(lat->d_col[1], (unsigned char)value, (size_t)(lat->N / 2), ctx->stream));
    if (lat->layout == MCX_LAYOUT_MSC64) MCX_CHECK(msc_pack(lat));
    return recompute_state(lat);
}

MCX_API mcx_status mcx_observables(mcx_lattice* lat, int64_t* pair_sum, int64_t* spin_sum,
                                   int64_t* spin2_sum) {
    if (!lat) return fail(MCX_ERR_INVALID_ARG, "lattice is NULL");
    int64_t st[3];
    MCX_CUDA(cudaMemcpyAsync(st, lat->d_state, sizeof(st), cudaMemcpyDeviceToHost, lat->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(lat->ctx->stream));
    if (pair_sum) *pair_sum = st[0];
    if (spin_sum) *spin_sum = st[1];
    if (spin2_sum) *spin2_sum = st[2];
    return MCX_OK;
}

MCX_API mcx_status mcx_recompute_observables(mcx_lattice* lat, int64_t* pair_sum, int64_t* spin_sum,
                                             int64_t* spin2_sum) {
    if (!lat) return fail(MCX_ERR_INVALID_ARG, "lattice is NULL");
    MCX_CHECK(recompute_state(lat));
    return mcx_observables(lat, pair_sum, spin_sum, spin2_sum);
}

MCX_API mcx_status mcx_energy(mcx_lattice* lat, double* energy, int64_t* magnetization) {
    int64_t P, M, Q;
    MCX_CHECK(mcx_observables(lat, &P, &M, &Q));
    // _cached_energy: -J*pair - h*M (+ D*Q for Blume-Capel), SpinSystems/src/ising.jl:181-183, :472, SpinSystems/src/blume_capel.jl:221-223
    double E = (-(lat->J * (double)P)) - (lat->h * (double)M);
    if (lat->model == MCX_BLUME_CAPEL) E = E + lat->D * (double)Q;
    if (energy) *energy = E;
    if (magnetization) *magnetization = M;
    return MCX_OK;
}

MCX_API mcx_status mcx_read_series(mcx_lattice* lat, int64_t* obs, int64_t n) {
    if (!lat || !obs) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (n < 0 || n > lat->series_len)
        return fail(MCX_ERR_INVALID_ARG, "requested %lld sweeps, %lld recorded", (long long)n,
                    (long long)lat->series_len);
    MCX_CUDA(cudaMemcpyAsync(obs, lat->d_series, (size_t)n * 3 * sizeof(int64_t), cudaMemcpyDeviceToHost,
                             lat->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(lat->ctx->stream));
    return MCX_OK;
}

}  // extern "C"

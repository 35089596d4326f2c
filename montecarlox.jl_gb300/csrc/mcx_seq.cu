// mcx_seq.cu -- the reference's own update order on a device lattice: `spin_flip!(sys, alg)`
// at a uniformly random site, one attempt after another (SpinSystems/src/abstractions.jl:19
// pick_site, SpinSystems/src/ising.jl:25-58, SpinSystems/src/blume_capel.jl:41-85), with the
// FP64 decisions of src/algorithms/importance_sampling.jl:80-85 (Metropolis, lr > 0 ||
// U < exp(lr)), src/algorithms/metropolis.jl:121-127 (Glauber, U < logistic(lr)) and the heat
// baths of ising.jl:43-58 / blume_capel.jl:61-85.
//
// Attempt a draws Philox4x32-10(key = seed, counter = (a lo, a hi, 5 << 24, stream)): the
// site is ((w0 << 32) | w1) mod N and U = u53(w2, w3); a Blume-Capel Metropolis / Glauber
// proposal takes the top bit of word 0 of the counter (a lo, a hi, 6 << 24, stream).
//
// The probabilities are FP64 values the host computes once per call with the reference's
// formulas in the reference's operation order (exp and logistic of the host C library), one
// per (spin, neighbour sum) state; the device only compares U against them, so each decision
// is the FP64 comparison the reference makes, bit for bit.
//
// The attempts are serial (each may read a spin the one before wrote).  One warp draws the
// random words of 32 attempts in parallel; one thread then applies them in order.  A lattice
// of at most kSeqSmemSites sites is held in shared memory for the call.
#include <cmath>
#include <cstring>

#include "mcx_device.cuh"
#include "mcx_internal.h"

namespace mcx {
mcx_status msc_pack(mcx_lattice* lat);
mcx_status msc_unpack(mcx_lattice* lat);
}  // namespace mcx

using namespace mcx;

namespace {

constexpr uint32_t P_SEQ = 5;
constexpr uint32_t P_SEQ2 = 6;
constexpr long long kSeqSmemSites = 196608;  // 192 KiB of shared memory
constexpr int kSeqThreads = 256;

// Ising: p[a + (z+1)*up], a = aligned neighbours; flip iff (U < p) != inv[...].
// Blume-Capel Metropolis / Glauber: p[(s+1)*2*nc + b*nc + (c+z)], accept iff U < p.
// Blume-Capel heat bath: w1[c+z], w12[c+z], zz[c+z]: r = U*zz, s = r < w1 ? -1 : r < w12 ? 0 : 1.
struct SeqTable {
    double p[78];
    double w1[13], w12[13], zz[13];
    unsigned char inv[14];
};

struct SeqGeo {
    int Lx, Ly, Lz, W;
    long long N;
};

// logistic, src/infrastructure/utils.jl:82-88
double logistic_h(double x) {
    if (x >= 0) return 1.0 / (1.0 + std::exp(-x));
    double ex = std::exp(x);
    return ex / (1.0 + ex);
}

// lr > 0 || U < exp(lr)  <=>  U < p with p = 2 for lr > 0 (U < 1 always)
double metropolis_p(double lr) { return lr > 0 ? 2.0 : std::exp(lr); }

int bc_propose_h(int s_old, int b) {  // _propose_state, SpinSystems/src/blume_capel.jl:21-30
    if (s_old == -1) return b ? 0 : 1;
    if (s_old == 0) return b ? -1 : 1;
    return b ? -1 : 0;
}

__device__ __forceinline__ int bc_propose_d(int s_old, int b) {
    if (s_old == -1) return b ? 0 : 1;
    if (s_old == 0) return b ? -1 : 1;
    return b ? -1 : 0;
}

mcx_status build_seq_table(const mcx_lattice* lat, mcx_algorithm alg, double beta, SeqTable* t) {
    const int z = 2 * lat->dim, nc = 2 * z + 1;
    const double J = lat->J, D = lat->D, h = lat->h;
    std::memset(t, 0, sizeof(*t));
    if (alg != MCX_METROPOLIS && alg != MCX_GLAUBER && alg != MCX_HEATBATH)
        return fail(MCX_ERR_INVALID_ARG, "unknown algorithm %d", (int)alg);
    if (lat->model == MCX_ISING) {
        for (int up = 0; up < 2; ++up)
            for (int a = 0; a <= z; ++a) {
                const double so = up ? 1.0 : -1.0;
                const double lpi = (double)(2 * a - z);     // s_i * sum of the neighbours
                const double dpair = ((-2.0) * J) * lpi;    // flip_changes, ising.jl:484-489
                const double dspin = -2.0 * so;
                const double dE = (-dpair) - (h * dspin);   // delta_energy
                double p;
                unsigned char inv = 0;
                if (alg == MCX_METROPOLIS) {
                    p = metropolis_p((-beta) * dE);
                } else if (alg == MCX_GLAUBER) {
                    p = logistic_h((-beta) * dE);
                } else {  // p_plus = logistic(beta*s_old*dE); s_new = U < p_plus ? +1 : -1
                    p = logistic_h((beta * so) * dE);
                    inv = (unsigned char)up;  // an up spin flips iff !(U < p_plus)
                }
                t->p[a + (z + 1) * up] = p;
                t->inv[a + (z + 1) * up] = inv;
            }
        return MCX_OK;
    }
    if (alg == MCX_HEATBATH) {
        for (int c = -z; c <= z; ++c) {
            const double coupling = J * (double)c;
            const double e1 = (coupling - (h * -1.0)) + D;
            const double e3 = ((-coupling) - (h * 1.0)) + D;
            const double w1 = std::exp((-beta) * e1), w2 = std::exp((-beta) * 0.0), w3 = std::exp((-beta) * e3);
            t->w1[c + z] = w1;
            t->w12[c + z] = w1 + w2;
            t->zz[c + z] = (w1 + w2) + w3;
        }
        return MCX_OK;
    }
    for (int so = -1; so <= 1; ++so)
        for (int b = 0; b < 2; ++b)
            for (int c = -z; c <= z; ++c) {
                const int sn = bc_propose_h(so, b);
                const double ds = (double)(sn - so), ds2 = (double)(sn * sn - so * so);
                const double dE = ((-(ds * (J * (double)c))) - (h * ds)) + (D * ds2);  // blume_capel.jl:247-248
                const double lr = (-beta) * dE;
                t->p[(so + 1) * 2 * nc + b * nc + (c + z)] = alg == MCX_METROPOLIS ? metropolis_p(lr) : logistic_h(lr);
            }
    return MCX_OK;
}

// spin at (x, y, z) of the colour-split arrays (colour (x+y+z)&1, row y + Ly z, entry x >> 1)
__device__ __forceinline__ long long seq_off(const SeqGeo& g, int x, int y, int z) {
    return ((long long)y + (long long)g.Ly * z) * g.W + (x >> 1);
}

template <int DIM, int MODEL>
__global__ void __launch_bounds__(kSeqThreads) k_seq(int8_t* __restrict__ c0, int8_t* __restrict__ c1, SeqGeo g,
                                                     SeqTable tab, int alg, uint32_t k0, uint32_t k1,
                                                     uint32_t stream, unsigned long long a0, long long n,
                                                     long long* __restrict__ state,
                                                     unsigned long long* __restrict__ counts, int use_smem) {
    extern __shared__ int8_t sm[];
    __shared__ long long s_site[32];
    __shared__ double s_u[32];
    __shared__ int s_b[32];
    const long long half = g.N / 2;
    int8_t* b0 = c0;
    int8_t* b1 = c1;
    if (use_smem) {
        for (long long k = threadIdx.x; k < half; k += blockDim.x) {
            sm[k] = c0[k];
            sm[half + k] = c1[k];
        }
        __syncthreads();
        b0 = sm;
        b1 = sm + half;
    }
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const int z = 2 * DIM, nc = 2 * z + 1;
        long long dp = 0, dm = 0, dq = 0;
        unsigned long long acc = 0;
        for (long long base = 0; base < n; base += 32) {
            const long long m = n - base < 32 ? n - base : 32;
            if (lane < m) {
                const unsigned long long a = a0 + (unsigned long long)(base + lane);
                const uint4 w = philox10(make_uint4((uint32_t)a, (uint32_t)(a >> 32), P_SEQ << 24, stream), k0, k1);
                s_site[lane] = (long long)((((unsigned long long)w.x << 32) | w.y) % (unsigned long long)g.N);
                s_u[lane] = u53(w.z, w.w);
                int b = 0;
                if (MODEL == MCX_BLUME_CAPEL && alg != MCX_HEATBATH)
                    b = (int)(philox10(make_uint4((uint32_t)a, (uint32_t)(a >> 32), P_SEQ2 << 24, stream), k0, k1).x >>
                              31);
                s_b[lane] = b;
            }
            __syncwarp();
            if (lane == 0) {
                for (int j = 0; j < (int)m; ++j) {
                    const long long i = s_site[j];
                    const double U = s_u[j];
                    const int x = (int)(i % g.Lx);
                    const long long rr = i / g.Lx;
                    const int y = (int)(rr % g.Ly);
                    const int zc = (int)(rr / g.Ly);
                    const int c = (x + y + zc) & 1;
                    int8_t* own = c ? b1 : b0;
                    const int8_t* oth = c ? b0 : b1;
                    const long long io = seq_off(g, x, y, zc);
                    const int so = own[io];
                    const int xp = x + 1 == g.Lx ? 0 : x + 1, xm = x == 0 ? g.Lx - 1 : x - 1;
                    const int yp = y + 1 == g.Ly ? 0 : y + 1, ym = y == 0 ? g.Ly - 1 : y - 1;
                    int S = oth[seq_off(g, xp, y, zc)] + oth[seq_off(g, xm, y, zc)] + oth[seq_off(g, x, yp, zc)] +
                            oth[seq_off(g, x, ym, zc)];
                    if (DIM == 3) {
                        const int zp = zc + 1 == g.Lz ? 0 : zc + 1, zm = zc == 0 ? g.Lz - 1 : zc - 1;
                        S += oth[seq_off(g, x, y, zp)] + oth[seq_off(g, x, y, zm)];
                    }
                    int sn = so;
                    if (MODEL == MCX_ISING) {
                        const int e = ((so * S + z) >> 1) + (z + 1) * (so > 0);
                        if ((U < tab.p[e]) != (tab.inv[e] != 0)) sn = -so;
                    } else if (alg == MCX_HEATBATH) {
                        const double r = U * tab.zz[S + z];
                        sn = r < tab.w1[S + z] ? -1 : (r < tab.w12[S + z] ? 0 : 1);
                    } else {
                        const int b = s_b[j];
                        const int prop = bc_propose_d(so, b);
                        if (U < tab.p[(so + 1) * 2 * nc + b * nc + (S + z)]) sn = prop;
                    }
                    if (sn != so) {
                        own[io] = (int8_t)sn;
                        dp += (long long)(sn - so) * S;
                        dm += sn - so;
                        dq += sn * sn - so * so;
                        ++acc;
                    }
                }
            }
            __syncwarp();
        }
        if (lane == 0) {
            state[0] += dp;
            state[1] += dm;
            state[2] += dq;
            counts[0] = (unsigned long long)n;
            counts[1] = acc;
        }
    }
    if (use_smem) {
        __syncthreads();
        for (long long k = threadIdx.x; k < half; k += blockDim.x) {
            c0[k] = sm[k];
            c1[k] = sm[half + k];
        }
    }
}

template <int DIM, int MODEL>
const void* seq_kernel() {
    return reinterpret_cast<const void*>(&k_seq<DIM, MODEL>);
}

}  // namespace

extern "C" {

// N x spin_flip!(sys, alg) in the reference's random-site order (declared in mcx.h).
MCX_API mcx_status mcx_spin_flip(mcx_lattice* lat, mcx_algorithm alg, double beta, mcx_rng* rng,
                                 int64_t nattempts, mcx_counters* counters) {
    if (!lat || !rng) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (nattempts < 0) return fail(MCX_ERR_INVALID_ARG, "nattempts must be >= 0");
    if (!std::isfinite(beta)) return fail(MCX_ERR_INVALID_ARG, "beta must be finite");
    if (nattempts == 0) return MCX_OK;
    SeqTable tab;
    MCX_CHECK(build_seq_table(lat, alg, beta, &tab));
    mcx_ctx* ctx = lat->ctx;
    if (lat->layout == MCX_LAYOUT_MSC64) MCX_CHECK(msc_unpack(lat));
    SeqGeo g;
    g.Lx = (int)lat->L[0];
    g.Ly = (int)lat->L[1];
    g.Lz = (int)lat->L[2];
    g.W = (int)lat->W;
    g.N = lat->N;
    const int use_smem = lat->N <= kSeqSmemSites ? 1 : 0;
    const size_t smem = use_smem ? (size_t)lat->N : 0;
    const void* fn = lat->dim == 2 ? (lat->model == MCX_ISING ? seq_kernel<2, MCX_ISING>() : seq_kernel<2, MCX_BLUME_CAPEL>())
                                   : (lat->model == MCX_ISING ? seq_kernel<3, MCX_ISING>() : seq_kernel<3, MCX_BLUME_CAPEL>());
    if (smem > 48 * 1024) MCX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    void* scratch = nullptr;  // (attempts, accepted) of this call
    MCX_CHECK(ctx_scratch(ctx, 2 * sizeof(unsigned long long), &scratch));
    unsigned long long* counts = static_cast<unsigned long long*>(scratch);
    int8_t* c0 = lat->d_col[0];
    int8_t* c1 = lat->d_col[1];
    int ialg = (int)alg;
    uint32_t k0 = (uint32_t)rng->seed, k1 = (uint32_t)(rng->seed >> 32), st = rng->stream;
    unsigned long long a0 = rng->counter;
    long long n = nattempts;
    long long* state = (long long*)lat->d_state;
    int smem_flag = use_smem;
    void* args[] = {&c0, &c1, &g, &tab, &ialg, &k0, &k1, &st, &a0, &n, &state, &counts, &smem_flag};
    MCX_CUDA(cudaLaunchKernel(fn, dim3(1), dim3(kSeqThreads), args, smem, ctx->stream));
    count_launch(ctx);
    if (lat->layout == MCX_LAYOUT_MSC64) MCX_CHECK(msc_pack(lat));
    rng->counter += (uint64_t)nattempts;
    if (counters) {
        unsigned long long h[2];
        MCX_CUDA(cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
        MCX_CUDA(cudaStreamSynchronize(ctx->stream));
        counters->attempts += h[0];
        counters->accepted += h[1];
    }
    return MCX_OK;
}

}  // extern "C"

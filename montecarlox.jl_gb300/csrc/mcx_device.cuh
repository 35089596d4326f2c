// mcx_device.cuh -- device helpers: Philox4x32-10, 53-bit uniforms, the project
// log, warp/block integer reductions.  Compiled with --fmad=false so that every
// FP64 expression is evaluated exactly as written.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace mcx {

__host__ __device__ __forceinline__ double bits_to_double(long long b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double d;
    std::memcpy(&d, &b, 8);
    return d;
#endif
}

__host__ __device__ __forceinline__ long long double_to_bits(double d) {
#ifdef __CUDA_ARCH__
    return __double_as_longlong(d);
#else
    long long b;
    std::memcpy(&b, &d, 8);
    return b;
#endif
}

constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11); also on the host, where the
// exchange decisions of a ladder spread over processes are taken.
__host__ __device__ __forceinline__ uint4 philox10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += kPhiloxW0;
            k1 += kPhiloxW1;
        }
        unsigned long long p0 = (unsigned long long)kPhiloxM0 * c.x;
        unsigned long long p1 = (unsigned long long)kPhiloxM1 * c.z;
        c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1,
                       (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0);
    }
    return c;
}

// philox10 for counters (x, y, z, w) of which only x and w vary between calls: the
// round-0 product of z and the round-1 product of the resulting first word do not depend
// on x or w, so they are formed once (philox_pre) and each call does 18 products, not 20.
// philox10_pre(x, w, philox_pre(y, z, k0), k0, k1) == philox10({x, y, z, w}, k0, k1).
struct PhiloxPre {
    uint32_t x1, y1;      // round-0 words 0 and 1
    uint32_t hi1, lo1;    // round-1 product of word 0
};

__host__ __device__ __forceinline__ PhiloxPre philox_pre(uint32_t y, uint32_t z, uint32_t k0) {
    const unsigned long long p1 = (unsigned long long)kPhiloxM1 * z;
    PhiloxPre P;
    P.x1 = (uint32_t)(p1 >> 32) ^ y ^ k0;
    P.y1 = (uint32_t)p1;
    const unsigned long long p0 = (unsigned long long)kPhiloxM0 * P.x1;
    P.hi1 = (uint32_t)(p0 >> 32);
    P.lo1 = (uint32_t)p0;
    return P;
}

__host__ __device__ __forceinline__ uint4 philox10_pre(uint32_t x, uint32_t w, const PhiloxPre& P, uint32_t k0,
                                                       uint32_t k1) {
    const unsigned long long q0 = (unsigned long long)kPhiloxM0 * x;  // round 0
    const uint32_t z1 = (uint32_t)(q0 >> 32) ^ w ^ k1, w1 = (uint32_t)q0;
    k0 += kPhiloxW0;  // round 1
    k1 += kPhiloxW1;
    const unsigned long long q1 = (unsigned long long)kPhiloxM1 * z1;
    uint4 c = make_uint4((uint32_t)(q1 >> 32) ^ P.y1 ^ k0, (uint32_t)q1, P.hi1 ^ w1 ^ k1, P.lo1);
#pragma unroll
    for (int r = 2; r < 10; ++r) {
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
        unsigned long long p0 = (unsigned long long)kPhiloxM0 * c.x;
        unsigned long long p1 = (unsigned long long)kPhiloxM1 * c.z;
        c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0);
    }
    return c;
}

// word 2 of a checkerboard counter
__host__ __device__ __forceinline__ uint32_t ctr_word2(unsigned long long sweep, int colour,
                                              uint32_t purpose) {
    return ((uint32_t)(sweep >> 32) & 0xFFFFu) | ((uint32_t)colour << 16) | (purpose << 24);
}

__device__ __forceinline__ uint32_t pick4(uint4 w, int lane) {
    return lane == 0 ? w.x : lane == 1 ? w.y : lane == 2 ? w.z : w.w;
}

__host__ __device__ __forceinline__ double u53(uint32_t hi, uint32_t lo) {
    unsigned long long k = ((unsigned long long)hi << 21) | (unsigned long long)(lo >> 11);
    return (double)k * 1.1102230246251565404236316680908203125e-16;  // 2^-53
}

// log(x) from log(m) = 2 atanh((m-1)/(m+1)) after x = 2^k m, m in [sqrt(1/2), sqrt(2)).
// Plain multiplies and adds, in a fixed order, so host and device agree bit for bit.
__host__ __device__ __forceinline__ double mcx_log(double x) {
    if (x != x) return x;
    if (x < 0.0) return bits_to_double(0x7FF8000000000000ll);
    if (x == 0.0) return bits_to_double(0xFFF0000000000000ll);
    if (x == bits_to_double(0x7FF0000000000000ll)) return x;
    long long b = double_to_bits(x);
    long long k = 0;
    if ((b >> 52) == 0) {
        double y = x * 18014398509481984.0;  // 2^54
        b = double_to_bits(y);
        k = -54;
    }
    k += (b >> 52) - 1023;
    double m = bits_to_double((b & 0x000FFFFFFFFFFFFFll) | 0x3FF0000000000000ll);
    if (m > 1.4142135623730951) {
        m = m * 0.5;
        k += 1;
    }
    double f = m - 1.0;
    double s = f / (m + 1.0);
    double s2 = s * s;
    double p = 1.0 / 23.0;
    p = p * s2 + 1.0 / 21.0;
    p = p * s2 + 1.0 / 19.0;
    p = p * s2 + 1.0 / 17.0;
    p = p * s2 + 1.0 / 15.0;
    p = p * s2 + 1.0 / 13.0;
    p = p * s2 + 1.0 / 11.0;
    p = p * s2 + 1.0 / 9.0;
    p = p * s2 + 1.0 / 7.0;
    p = p * s2 + 1.0 / 5.0;
    p = p * s2 + 1.0 / 3.0;
    double two_s = s + s;
    double lm = two_s + two_s * (s2 * p);
    double kd = (double)k;
    const double ln2_hi = 6.93147180369123816490e-01;
    const double ln2_lo = 1.90821492927058770002e-10;
    return kd * ln2_hi + (lm + kd * ln2_lo);
}

// exp(x): Cody & Waite argument reduction x = k ln2 + r, |r| <= ln2/2, with ln2 split
// into a 32-bit head (k * head is exact) and a tail; exp(r) from its Taylor series up to
// r^13/13! in Horner form; then 2^k is put in with one or two exact scalings.  Plain
// multiplies and adds in a fixed order, so host and device agree bit for bit.
__host__ __device__ __forceinline__ double mcx_pow2(int k) {  // 2^k, -1022 <= k <= 1023
    return bits_to_double((long long)(k + 1023) << 52);
}

__host__ __device__ __forceinline__ double mcx_exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return bits_to_double(0x7FF0000000000000ll);
    if (x < -745.2) return 0.0;
    const double kd = floor(x * 0x1.71547652b82fep+0 + 0.5);
    const double r = (x - kd * 0x1.62e42fee00000p-1) - kd * 0x1.a39ef35793c76p-33;
    double p = 0x1.6124613a86d09p-33;
    p = p * r + 0x1.1eed8eff8d898p-29;
    p = p * r + 0x1.ae64567f544e4p-26;
    p = p * r + 0x1.27e4fb7789f5cp-22;
    p = p * r + 0x1.71de3a556c734p-19;
    p = p * r + 0x1.a01a01a01a01ap-16;
    p = p * r + 0x1.a01a01a01a01ap-13;
    p = p * r + 0x1.6c16c16c16c17p-10;
    p = p * r + 0x1.1111111111111p-7;
    p = p * r + 0x1.5555555555555p-5;
    p = p * r + 0x1.5555555555555p-3;
    p = p * r + 0.5;
    p = p * r + 1.0;
    p = p * r + 1.0;
    const int k = (int)kd;
    if (k > 1023) return (p * mcx_pow2(k - 1)) * 2.0;
    if (k < -1021) return (p * mcx_pow2(k + 64)) * 0x1p-64;
    return p * mcx_pow2(k);
}

// logistic(x), src/infrastructure/utils.jl:82-88, on mcx_exp
__host__ __device__ __forceinline__ double mcx_logistic(double x) {
    if (x >= 0) return 1.0 / (1.0 + mcx_exp(-x));
    const double ex = mcx_exp(x);
    return ex / (1.0 + ex);
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier of a cooperative launch with a bounded wait: bar[0] arrivals,
// bar[1] generation, bar[2] error flag.  A wait that exceeds `limit` polls sets the error
// flag; every block then leaves at its next barrier and the host reports MCX_ERR_TIMEOUT.
// The gpu-scope acquire of the generation orders the block's later loads after every
// other block's writes before the barrier.
__device__ __forceinline__ bool grid_sync(unsigned* bar, unsigned nblocks, unsigned& gen, long long limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        const unsigned g = gen;
        if (atomicAdd(&bar[0], 1u) == nblocks - 1) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            st_release(&bar[1], g + 1);
        } else {
            long long n = 0;
            while (ld_acquire(&bar[1]) == g) {
                if (ld_acquire(&bar[2]) != 0u) { ok = 0; break; }
                if (++n > limit) { atomicExch(&bar[2], 1u); ok = 0; break; }
                __nanosleep(100);
            }
        }
        gen = g + 1;
        s_ok = ok && ld_acquire(&bar[2]) == 0u;
    }
    __syncthreads();
    return s_ok != 0;
}

// Block-wide sum of up to 4 int64 values, one atomicAdd per value per block.
template <int NV>
__device__ __forceinline__ void block_add_atomic(long long (&v)[NV], unsigned long long* const (&dst)[NV]) {
    __shared__ long long red[32][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        long long x = v[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
        if (lane == 0) red[warp][j] = x;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            long long x = lane < nw ? red[lane][j] : 0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xFFFFFFFFu, x, o);
            if (lane == 0 && x != 0 && dst[j] != nullptr) atomicAdd(dst[j], (unsigned long long)x);
        }
    }
    __syncthreads();
}

// Programmatic dependent launch (PTX griddepcontrol, sm_90 and later).  pdl_wait blocks
// until the grid this launch depends on has completed and its memory operations are
// visible (it returns at once for a launch made without that dependency); pdl_trigger lets
// the dependent launch be scheduled before this grid ends.  A kernel reads nothing another
// kernel writes before pdl_wait.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Warp-wide sum of up to 4 values, one atomicAdd per nonzero value per warp, no barrier.
// The caller guarantees that every per-warp sum fits in int32 (the small-lattice bodies:
// at most 64 sites per thread and sweep, each changing a count by at most 12).
template <int NV>
__device__ __forceinline__ void warp_add_atomic(const long long (&v)[NV], unsigned long long* const (&dst)[NV]) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        int x = (int)v[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xFFFFFFFFu, x, o);
        if ((threadIdx.x & 31) == 0 && x != 0 && dst[j] != nullptr)
            atomicAdd(dst[j], (unsigned long long)(long long)x);
    }
}

}  // namespace mcx

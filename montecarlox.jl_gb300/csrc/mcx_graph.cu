// mcx_graph.cu -- Ising models on general neighbour lists: IsingGraph (one coupling over a
// graph, SpinSystems/src/ising.jl:86-218) and IsingMatrix (symmetric sparse J_ij,
// ising.jl:221-377), with no field, a uniform field or a field per site.
//
// Layout in HBM.  Sites are renumbered by colour class (first-fit colouring in vertex
// order; inside a class in vertex order) and every class is padded to a multiple of 32
// with dummy sites of spin 0 and no neighbours.  The neighbour lists are stored
// sliced-ELL: 32 consecutive positions form a slice whose entries are stored column-major
// -- entry k of lane l at soff[s] + 32k + l, padded with -1 to the longest list of the
// slice -- so that a warp reads one slice per step and every load of a neighbour position
// (and of a per-entry coupling) is a single coalesced transaction.  The spins of the other
// classes are gathered through the L2 (one byte per site; a 16M-site graph is 16 MB).
//
// Decisions are the reference's FP64 rules.  With one coupling and no per-site field,
// ΔE depends only on (s_i, Σ_j s_i s_j), so the host tabulates, per (s_i, lpi), the
// 53-bit integer threshold T = ceil(p 2^53) with u < p  <=>  k < T for u = k 2^-53: the
// device decision is then one 64-bit integer compare, identical to the FP64 one.
// Otherwise every site evaluates ΔE, exp and logistic in FP64 with the library's own
// mcx_exp (bit-identical on host and device).
#include <algorithm>
#include <cmath>
#include <vector>

#include "mcx_device.cuh"
#include "mcx_internal.h"

using namespace mcx;

namespace {

constexpr int kGraphBlock = 256;
constexpr int kSlicesPerBlock = kGraphBlock / 32;
constexpr int small_block(bool table) { return table ? 1024 : 512; }
constexpr long long kSmallGraph = 8192;  // padded positions run by the one-block kernel
constexpr int kMaxTableDegree = 4096;
constexpr unsigned long long kAlways53 = (1ull << 53) + 1;

enum GField { F_NONE = 0, F_UNIFORM = 1, F_VECTOR = 2 };

struct GraphDev {
    int8_t* spins;                  // padded positions, renumbered order
    const int32_t* nbr;             // sliced-ELL neighbour positions (-1 = padding)
    const double* J64;              // per entry (IsingMatrix), or nullptr
    const float2* J2;               // the same couplings split hi + lo, or nullptr
    const long long* soff;          // nslices + 1 entry offsets
    const double* h;                // per position (vector field), or nullptr
    const float2* h2;               // the same split hi + lo, or nullptr
    double J, hu;                   // uniform coupling, uniform field
    float2 J2u, h2u, D2u;           // the same split hi + lo (and the crystal field)
    const unsigned long long* tab;  // thresholds by (s > 0, lpi + dmax)
    const float2* tabdE;            // ΔE (hi + lo) by (s > 0, lpi + dmax)
    int dmax;
    double beta;
    float beta32;
    double D;                       // crystal field (Blume-Capel)
    unsigned long long* acc;        // accepted moves
    long long* M;                   // cached magnetization
    double* E;                      // cached energy
    double* part;                   // per-block partial sums of ΔE
};

struct GClass {
    long long p0;       // first padded position of the class
    long long count;    // sites of the class
    long long blk0;     // first Philox block of the class
    long long slice0;   // first slice
    long long nslices;
    int part0;          // first partial-sum slot
};

// Deterministic block sum of one FP64 value (fixed shuffle tree, then warps in order);
// the result is valid in thread 0.
__device__ __forceinline__ double block_sum_f64(double v) {
    __shared__ double red[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    __syncthreads();
    return t;
}

__device__ __forceinline__ long long warp_sum_i64(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Float-float accumulation (s_hi, s_lo) += (x_hi, x_lo): Knuth's two-sum of the high
// parts, the low parts added to its error, then a fast renormalisation.
__device__ __forceinline__ void ff_add(float& sh, float& sl, float xh, float xl) {
    const float t = sh + xh;
    const float bb = t - sh;
    const float e = (sh - (t - bb)) + (xh - bb);
    const float u = e + (sl + xl);
    sh = t + u;
    sl = u - (sh - t);
}

// ΔE of the site at padded position p in FP64 exactly as the reference: flip_changes +
// delta_energy, -Δpair - h Δspin with Δpair = -2 acc (IsingMatrix, acc the sequential
// FP64 sum of s_i J_ij s_j over the row) or -2 J lpi (IsingGraph), Δspin = -2 s.
template <bool EDGEJ, int FIELD>
__device__ __forceinline__ double site_delta_energy(const GraphDev& g, const int8_t* sp, long long p, long long off,
                                                    int w, int lane, int si, int lpi) {
    double dpair;
    if (EDGEJ) {
        double acc = 0.0;
        for (int k = 0; k < w; ++k) {
            const long long e = off + 32ll * k + lane;
            const int nb = g.nbr[e];
            if (nb >= 0) {
                const double Jk = g.J64[e];
                acc += (si * sp[nb] > 0) ? Jk : -Jk;  // (s_i J) s_j: exact sign flips
            }
        }
        dpair = -2.0 * acc;
    } else {
        dpair = (-2.0 * g.J) * (double)lpi;
    }
    const double dspin = (double)(-2 * si);
    if (FIELD == F_VECTOR) return -dpair - g.h[p] * dspin;
    if (FIELD == F_UNIFORM) return -dpair - g.hu * dspin;
    return -dpair;
}

// The reference's FP64 decision for one site (the exact path, taken when the FP32 test
// below cannot decide).  Returns the flip and ΔE.
template <int ALG, bool EDGEJ, int FIELD>
__device__ __noinline__ bool exact_site(const GraphDev& g, const int8_t* sp, long long p, long long off, int w,
                                        int lane, int si, int lpi, unsigned long long ku, double* dE_out) {
    const double dE = site_delta_energy<EDGEJ, FIELD>(g, sp, p, off, w, lane, si, lpi);
    *dE_out = dE;
    const double u = (double)ku * 0x1p-53;
    if (ALG == MCX_METROPOLIS) {
        const double lr = -g.beta * dE;
        return (lr > 0) || (u < mcx_exp(lr));
    }
    if (ALG == MCX_GLAUBER) return u < mcx_logistic(-g.beta * dE);
    const bool up = u < mcx_logistic((g.beta * (double)si) * dE);
    return up != (si == 1);
}

// Certified FP32 decision of "u < p" where p = exp(x) (Metropolis, x <= 0 or accept) or
// p = logistic(x), x the FP64 argument of the reference and xf an FP32 estimate with
// |xf - x| <= errx.  u = w0 2^-32 + (low bits) >= w0 2^-32 and < (w0+1) 2^-32.  With
// pe the fast estimate of p -- __expf errs by at most 2 + 1.173 |x| ulp (CUDA programming
// guide), the FP32 addition and division by half an ulp each -- every p compatible with
// the bounds lies in pe (1 -+ m), m taken with a factor 2 or more on each term.  Returns
// 1 (u < p for sure), 0 (u >= p for sure) or -1 (undecided).  Outputs of __expf that
// flush to 0 or overflow leave pe = 0 (p below 2^-120: only w0 = 0 stays undecided) or
// pe = 1 (p above 1 - 2^-120).
template <bool LOGISTIC>
__device__ __forceinline__ int certain_below(float xf, float errx, uint32_t w0) {
    const float m = errx * 1.01f + fabsf(xf) * 0x1p-22f + 0x1p-19f;
    if (!(m < 0x1p-8f)) return -1;
    float pe;
    if (LOGISTIC) {
        pe = 1.0f / (1.0f + __expf(-xf));
    } else {
        if (xf > errx) return 1;  // x > 0: always accepted
        pe = __expf(fminf(xf, 0.0f));
    }
    const float A = pe * (1.0f - 2.0f * m) * 4294967296.0f;
    const uint32_t a = A >= 4294967040.0f ? 4294967040u : (uint32_t)A;
    if (w0 < a) return 1;
    const float B = pe * (1.0f + 2.0f * m) * 4294967296.0f;
    if (B >= 4294967040.0f) return -1;
    const uint32_t b = max((uint32_t)ceilf(B), 1u);
    return w0 >= b ? 0 : -1;
}

// Row sums of one site: the integer lpi (IsingGraph) or the float-float sum of
// s_i J_ij s_j from the split couplings with the bound S = Σ |J_hi| (IsingMatrix).
struct RowSum {
    int lpi;
    float ah, al, S;
};

// One site: ΔE in float-float, the certified FP32 decision, the exact FP64 one when that
// cannot decide.  Returns the flip; (eh, el) accumulates ΔE of flipped sites.
template <int ALG, bool TABLE, bool EDGEJ, int FIELD>
__device__ __forceinline__ bool decide_site(const GraphDev& g, const int8_t* sp, long long p, long long off, int w,
                                            int lane, int si, const RowSum& r, uint32_t whi, uint32_t wlo, float& eh,
                                            float& el) {
    const unsigned long long ku = ((unsigned long long)whi << 21) | (unsigned long long)(wlo >> 11);
    if (TABLE) {
        const int idx = (si > 0 ? 2 * g.dmax + 1 : 0) + r.lpi + g.dmax;
        const bool below = ku < g.tab[idx];
        const bool flip = ALG == MCX_HEATBATH ? (below != (si == 1)) : below;
        if (flip) {
            const float2 d = g.tabdE[idx];
            ff_add(eh, el, d.x, d.y);
        }
        return flip;
    }
    // ΔE = 2 acc + 2 s h (acc = Σ s_i J_ij s_j or J lpi) as float-float
    float dh, dl, S;
    if (EDGEJ) {
        dh = 2.0f * r.ah;
        dl = 2.0f * r.al;
        S = r.S;
    } else {
        const float lf = (float)r.lpi, j2 = 2.0f * g.J2u.x;
        dh = lf * j2;
        dl = __fmaf_rn(lf, j2, -dh) + lf * (2.0f * g.J2u.y);
        S = fabsf(dh);
    }
    float hm = 0.0f;
    if (FIELD != F_NONE) {
        const float2 hv = FIELD == F_VECTOR ? g.h2[p] : g.h2u;
        const float sg = (float)(2 * si);
        ff_add(dh, dl, sg * hv.x, sg * hv.y);
        hm = fabsf(hv.x);
    }
    // |df - ΔE_FP64| <= errd: df rounds the float-float value (2^-24 |df|); the float-float
    // row sum is within 2 (w+1)^2 2^-48 S of the exact one (the low word collects up to w
    // two-sum errors of at most 2^-24 S each, each addition rounding it by 2^-24); the FP64
    // reference sum is within w 2^-52 (2S + 2|h|) of the exact one.
    const float df = dh + dl;
    const float wf = (float)(w + 1);
    const float errd = (2.0f * S + 2.0f * hm + fabsf(df)) * 0x1p-20f + wf * wf * S * 0x1p-46f;
    float xf;
    if (ALG == MCX_HEATBATH) xf = (g.beta32 * (float)si) * df;
    else xf = -g.beta32 * df;
    const float errx = fabsf(g.beta32) * errd * 1.01f + fabsf(xf) * 0x1p-21f + 0x1p-126f;
    const int c = certain_below<ALG != MCX_METROPOLIS>(xf, errx, whi);
    bool flip;
    if (c >= 0) {
        flip = ALG == MCX_HEATBATH ? ((c == 1) != (si == 1)) : c == 1;
        if (flip) ff_add(eh, el, dh, dl);
    } else {
        double dE;
        flip = exact_site<ALG, EDGEJ, FIELD>(g, sp, p, off, w, lane, si, r.lpi, ku, &dE);
        if (flip) {
            const float h = __double2float_rn(dE);
            ff_add(eh, el, h, __double2float_rn(dE - (double)h));
        }
    }
    return flip;
}

// Both rows of a slice pair, four entries of each at a time: all index and coupling
// loads of a group are issued before any spin is gathered, and all gathers before any is
// used (each row keeps its own order).  NC: gather the spins through the read-only path,
// valid when no spin of another class changes during the launch.
template <bool EDGEJ, bool NC>
__device__ __forceinline__ void row_sum2(const GraphDev& g, const int8_t* sp, long long offA, int wA, long long offB,
                                         int wB, int lane, int siA, int siB, RowSum& rA, RowSum& rB) {
    rA.lpi = rB.lpi = 0;
    rA.ah = rA.al = rA.S = rB.ah = rB.al = rB.S = 0.0f;
    const int wm = max(wA, wB);
    for (int k = 0; k < wm; k += 4) {
        int na[4], nb[4];
        float2 Ja[4], Jb[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const long long ea = offA + 32ll * (k + j) + lane, eb = offB + 32ll * (k + j) + lane;
            na[j] = k + j < wA ? __ldg(g.nbr + ea) : -1;
            nb[j] = k + j < wB ? __ldg(g.nbr + eb) : -1;
            if (EDGEJ) {
                Ja[j] = k + j < wA ? __ldg(g.J2 + ea) : make_float2(0.0f, 0.0f);
                Jb[j] = k + j < wB ? __ldg(g.J2 + eb) : make_float2(0.0f, 0.0f);
            }
        }
        int sa[4], sb[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            sa[j] = na[j] >= 0 ? (int)(NC ? __ldg(sp + na[j]) : sp[na[j]]) : 0;
            sb[j] = nb[j] >= 0 ? (int)(NC ? __ldg(sp + nb[j]) : sp[nb[j]]) : 0;
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            RowSum& r = h ? rB : rA;
            const int si = h ? siB : siA;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int nj = h ? nb[j] : na[j];
                const int sj = h ? sb[j] : sa[j];
                if (EDGEJ) {
                    if (nj >= 0) {
                        const float2 Jk = h ? Jb[j] : Ja[j];
                        const bool pos = si * sj > 0;
                        const float xh = pos ? Jk.x : -Jk.x;
                        const float xl = pos ? Jk.y : -Jk.y;
                        const float t = r.ah + xh;
                        const float bb = t - r.ah;
                        r.al += ((r.ah - (t - bb)) + (xh - bb)) + xl;
                        r.ah = t;
                        r.S += fabsf(Jk.x);
                    }
                } else {
                    r.lpi += si * sj;
                }
            }
        }
    }
}

// row_sum2 for two rows of the same compile-time width (four neighbours: every torus in
// 2-D): no bounds test per entry (measured 7 % faster on the 4096^2 torus)
template <bool EDGEJ, bool NC, int WF>
__device__ __forceinline__ void row_sum2f(const GraphDev& g, const int8_t* sp, long long offA, int wA, long long offB,
                                         int wB, int lane, int siA, int siB, RowSum& rA, RowSum& rB) {
    rA.lpi = rB.lpi = 0;
    rA.ah = rA.al = rA.S = rB.ah = rB.al = rB.S = 0.0f;
    for (int k = 0; k < WF; k += 4) {
        int na[4], nb[4];
        float2 Ja[4], Jb[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const long long ea = offA + 32ll * (k + j) + lane, eb = offB + 32ll * (k + j) + lane;
            na[j] = __ldg(g.nbr + ea);
            nb[j] = __ldg(g.nbr + eb);
            if (EDGEJ) {
                Ja[j] = __ldg(g.J2 + ea);
                Jb[j] = __ldg(g.J2 + eb);
            }
        }
        int sa[4], sb[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            sa[j] = na[j] >= 0 ? (int)(NC ? __ldg(sp + na[j]) : sp[na[j]]) : 0;
            sb[j] = nb[j] >= 0 ? (int)(NC ? __ldg(sp + nb[j]) : sp[nb[j]]) : 0;
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            RowSum& r = h ? rB : rA;
            const int si = h ? siB : siA;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int nj = h ? nb[j] : na[j];
                const int sj = h ? sb[j] : sa[j];
                if (EDGEJ) {
                    if (nj >= 0) {
                        const float2 Jk = h ? Jb[j] : Ja[j];
                        const bool pos = si * sj > 0;
                        const float xh = pos ? Jk.x : -Jk.x;
                        const float xl = pos ? Jk.y : -Jk.y;
                        const float t = r.ah + xh;
                        const float bb = t - r.ah;
                        r.al += ((r.ah - (t - bb)) + (xh - bb)) + xl;
                        r.ah = t;
                        r.S += fabsf(Jk.x);
                    }
                } else {
                    r.lpi += si * sj;
                }
            }
        }
    }
}

// The slice pairs j = first, first + stride, ... of one colour class.  Pair j holds slices
// 2j and 2j+1 of the class; lane l draws one Philox block, blk0 + 32 j + l, whose words 0-1
// feed its site in slice 2j and words 2-3 its site in slice 2j+1.
template <int ALG, bool TABLE, bool EDGEJ, int FIELD, bool NC>
__device__ __forceinline__ void class_pairs(const GraphDev& g, int8_t* sp, const GClass& c, long long first,
                                            long long stride,
                                            int lane, uint32_t k0, uint32_t k1, uint32_t stream,
                                            unsigned long long sweep, float& eh, float& el, long long& dM,
                                            long long& nacc) {
    const uint32_t w2 = ctr_word2(sweep, 0, P_GRAPH);
    const long long npairs = (c.nslices + 1) >> 1;
    for (long long j = first; j < npairs; j += stride) {
        const long long sA = c.slice0 + 2 * j;
        const bool hasB = 2 * j + 1 < c.nslices;
        const long long pA = sA * 32 + lane, pB = pA + 32;
        const long long lA = 64 * j + lane, lB = lA + 32;  // class-local indices
        // slice sA + 1 exists (it is slice B or the first of the next class or the end mark)
        const long long offA = g.soff[sA], offB = g.soff[sA + 1];
        const int wA = (int)((offB - offA) >> 5);
        const int wB = hasB ? (int)((g.soff[sA + 2] - offB) >> 5) : 0;
        const int siA = sp[pA];
        const int siB = hasB ? (int)sp[pB] : 0;
        RowSum rA, rB;
        if (wA == 4 && wB == 4) row_sum2f<EDGEJ, NC, 4>(g, sp, offA, wA, offB, wB, lane, siA, siB, rA, rB);
        else row_sum2<EDGEJ, NC>(g, sp, offA, wA, offB, wB, lane, siA, siB, rA, rB);
        const uint4 r = philox10(make_uint4((uint32_t)(c.blk0 + 32 * j + lane), (uint32_t)sweep, w2, stream), k0, k1);
        if (lA < c.count) {
            if (decide_site<ALG, TABLE, EDGEJ, FIELD>(g, sp, pA, offA, wA, lane, siA, rA, r.x, r.y, eh, el)) {
                sp[pA] = (int8_t)(-siA);
                dM += -2 * siA;
                ++nacc;
            }
        }
        if (lB < c.count) {
            if (decide_site<ALG, TABLE, EDGEJ, FIELD>(g, sp, pB, offB, wB, lane, siB, rB, r.z, r.w, eh, el)) {
                sp[pB] = (int8_t)(-siB);
                dM += -2 * siB;
                ++nacc;
            }
        }
    }
}

// One colour class of one sweep over the whole grid.  The kernel waits on gathers: the
// FP32 path is held to 64 registers (4 blocks of 256 per SM), which measured faster than
// fewer, fatter warps; the table path needs 48.
template <int ALG, bool TABLE, bool EDGEJ, int FIELD>
__global__ void __launch_bounds__(kGraphBlock, TABLE ? 5 : 4) k_graph_class(GraphDev g, GClass c, uint32_t k0, uint32_t k1,
                                                             uint32_t stream, unsigned long long sweep) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    pdl_trigger();
    pdl_wait();  // the previous class (or sweep) is complete
    float eh = 0.0f, el = 0.0f;
    long long dM = 0;
    long long nacc = 0;
    class_pairs<ALG, TABLE, EDGEJ, FIELD, true>(g, g.spins, c, (long long)blockIdx.x * kSlicesPerBlock + warp,
                                                 (long long)gridDim.x * kSlicesPerBlock, lane, k0, k1, stream, sweep,
                                                 eh, el, dM, nacc);
    const double t = block_sum_f64((double)eh + (double)el);
    if (threadIdx.x == 0) g.part[c.part0 + blockIdx.x] = t;
    dM = warp_sum_i64(dM);
    nacc = warp_sum_i64(nacc);
    if (lane == 0) {
        if (dM) atomicAdd(reinterpret_cast<unsigned long long*>(g.M), (unsigned long long)dM);
        if (nacc) atomicAdd(g.acc, (unsigned long long)nacc);
    }
}

__device__ __forceinline__ void warp_ff_sum(float& h, float& l) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_down_sync(0xFFFFFFFFu, h, o), ol = __shfl_down_sync(0xFFFFFFFFu, l, o);
        ff_add(h, l, oh, ol);
    }
}

// Small graphs (up to kSmallGraph padded sites): every sweep of the call in one block
// (1024 threads for the table form; 512 for the FP32 form, whose sites need more than 64
// registers).  The spins live in shared memory for the whole call (a class reads what
// the previous one wrote, with a __syncthreads between classes); E, M and the accepted
// count stay in thread 0's registers; the per-sweep ΔE is reduced in float-float by
// shuffles (fixed order) and added to the FP64 energy once per sweep.  One launch per
// call instead of (classes + 1) per sweep.
template <int ALG, bool TABLE, bool EDGEJ, int FIELD>
__global__ void __launch_bounds__(small_block(TABLE), 1) k_graph_small(GraphDev g, const GClass* __restrict__ classes,
                                                                int ncls, uint32_t k0, uint32_t k1, uint32_t stream,
                                                                unsigned long long sweep0, long long nsweeps,
                                                                double* Eser, long long* Mser, int npad) {
    extern __shared__ int8_t s_spins[];
    __shared__ float red_f[2][32];
    __shared__ long long red_i[2][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (int)(blockDim.x >> 5);
    for (int p = threadIdx.x; p < npad; p += blockDim.x) s_spins[p] = g.spins[p];
    double E = 0.0;
    long long M = 0, acc = 0;
    if (threadIdx.x == 0) {
        E = *g.E;
        M = *g.M;
    }
    __syncthreads();
    for (long long t = 0; t < nsweeps; ++t) {
        float eh = 0.0f, el = 0.0f;
        long long dM = 0, nacc = 0;
        for (int k = 0; k < ncls; ++k) {
            class_pairs<ALG, TABLE, EDGEJ, FIELD, false>(g, s_spins, classes[k], warp, nw, lane, k0, k1, stream,
                                                          sweep0 + (unsigned long long)t, eh, el, dM, nacc);
            __syncthreads();
        }
        warp_ff_sum(eh, el);
        dM = warp_sum_i64(dM);
        nacc = warp_sum_i64(nacc);
        if (lane == 0) {
            red_f[0][warp] = eh;
            red_f[1][warp] = el;
            red_i[0][warp] = dM;
            red_i[1][warp] = nacc;
        }
        __syncthreads();
        if (warp == 0) {
            float h = lane < nw ? red_f[0][lane] : 0.0f, l = lane < nw ? red_f[1][lane] : 0.0f;
            long long m = lane < nw ? red_i[0][lane] : 0, a = lane < nw ? red_i[1][lane] : 0;
            warp_ff_sum(h, l);
            m = warp_sum_i64(m);
            a = warp_sum_i64(a);
            if (lane == 0) {
                E = E + ((double)h + (double)l);
                M += m;
                acc += a;
                if (Eser) Eser[t] = E;
                if (Mser) Mser[t] = M;
            }
        }
        __syncthreads();  // red_* are reused by the next sweep
    }
    for (int p = threadIdx.x; p < npad; p += blockDim.x) g.spins[p] = s_spins[p];
    if (threadIdx.x == 0) {
        *g.E = E;
        *g.M = M;
        *g.acc = *g.acc + (unsigned long long)acc;
    }
}

// ------------------------------------------------------------ Blume-Capel --
// BlumeCapelGraph / BlumeCapelMatrix (SpinSystems/src/blume_capel.jl:117-466): spins in
// {-1, 0, 1}, the same colour classes, slice pairs and Philox blocks as the Ising graphs.
// Metropolis / Glauber propose one of the two other states from bit 0 of the low word of
// the site's uniform (a bit the 53-bit uniform does not use); the heat bath draws from the
// three Boltzmann weights.  With one J and no per-site field the host tabulates exact
// 53-bit thresholds (for the heat bath the smallest k with fl(fl(k 2^-53) z) >= w, found
// by bisection on the reference's own FP64 expression r = u z < w); otherwise every site
// is evaluated in FP64 as the reference does.

// _propose_state, blume_capel.jl:21-30
__host__ __device__ __forceinline__ int bc_propose_state(int so, int b) {
    return so == -1 ? (b ? 0 : 1) : (so == 0 ? (b ? -1 : 1) : (b ? -1 : 0));
}

// propose_changes + delta_energy (:235-241, :247-248): -Δspin c - h Δspin + D Δspin2
__host__ __device__ __forceinline__ double bc_delta(double c, int so, int sn, double hf, bool field, double D) {
    const int ds = sn - so, ds2 = sn * sn - so * so;
    const double dpair = (double)ds * c;
    const double dfield = field ? hf * (double)ds : 0.0;
    return (-dpair - dfield) + D * (double)ds2;
}

// local_coupling (:227-229, :368-377): the integer neighbour sum and, for per-entry
// couplings, the FP64 sum of J_ij s_j in row order; four entries at a time.
template <bool EDGEJ>
__device__ __forceinline__ void bc_row(const GraphDev& g, const int8_t* sp, long long off, int w, int lane, int& isum,
                                       double& c) {
    isum = 0;
    c = 0.0;
    for (int k = 0; k < w; k += 4) {
        int nb[4];
        double Jk[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const long long e = off + 32ll * (k + j) + lane;
            nb[j] = k + j < w ? __ldg(g.nbr + e) : -1;
            if (EDGEJ) Jk[j] = k + j < w ? __ldg(g.J64 + e) : 0.0;
        }
        int sj[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) sj[j] = nb[j] >= 0 ? (int)sp[nb[j]] : 0;
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (nb[j] >= 0) {
                isum += sj[j];
                if (EDGEJ) c += Jk[j] * (double)sj[j];
            }
    }
}

// Float-float form of the coupling sum for the FP32 test: (ch, cl) = Σ J_ij s_j (or
// J Σ s_j) and S = Σ |J_ij| over the neighbours that are not 0 (|c| <= S).
struct BcRowFF {
    int isum;
    float ch, cl, S;
};

template <bool EDGEJ>
__device__ __forceinline__ void bc_row_ff(const GraphDev& g, const int8_t* sp, long long off, int w, int lane,
                                          BcRowFF& r) {
    r.isum = 0;
    r.ch = r.cl = r.S = 0.0f;
    for (int k = 0; k < w; k += 4) {
        int nb[4];
        float2 Jk[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const long long e = off + 32ll * (k + j) + lane;
            nb[j] = k + j < w ? __ldg(g.nbr + e) : -1;
            if (EDGEJ) Jk[j] = k + j < w ? __ldg(g.J2 + e) : make_float2(0.0f, 0.0f);
        }
        int sj[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) sj[j] = nb[j] >= 0 ? (int)sp[nb[j]] : 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            r.isum += sj[j];
            if (EDGEJ && sj[j] != 0) {
                const float xh = sj[j] > 0 ? Jk[j].x : -Jk[j].x, xl = sj[j] > 0 ? Jk[j].y : -Jk[j].y;
                const float t = r.ch + xh;
                const float bb = t - r.ch;
                r.cl += ((r.ch - (t - bb)) + (xh - bb)) + xl;
                r.ch = t;
                r.S += fabsf(Jk[j].x);
            }
        }
    }
    if (!EDGEJ) {
        const float lf = (float)r.isum;
        r.ch = lf * g.J2u.x;
        r.cl = __fmaf_rn(lf, g.J2u.x, -r.ch) + lf * g.J2u.y;
        r.S = fabsf(r.ch);
    }
}

// "u < p" from an FP32 estimate pe of p with every p compatible with the bounds in
// pe (1 -+ m): 1 sure, 0 surely not, -1 undecided (as certain_below).
__device__ __forceinline__ int certain_u(float pe, float m, uint32_t w0) {
    const float A = pe * (1.0f - 2.0f * m) * 4294967296.0f;
    const uint32_t a = A >= 4294967040.0f ? 4294967040u : (uint32_t)A;
    if (w0 < a) return 1;
    const float B = pe * (1.0f + 2.0f * m) * 4294967296.0f;
    if (B >= 4294967040.0f) return -1;
    const uint32_t b = max((uint32_t)ceilf(B), 1u);
    return w0 >= b ? 0 : -1;
}

// (dh, dl) = -ds c - ds h + ds2 D in float-float (|ds| <= 2, ds2 in {-1, 0, 1}: the
// products are exact)
template <int FIELD>
__device__ __forceinline__ void bc_delta_ff(const BcRowFF& r, float2 hv, float2 Dv, int ds, int ds2, float& dh,
                                            float& dl) {
    const float m = (float)(-ds);
    dh = m * r.ch;
    dl = m * r.cl;
    if (FIELD != F_NONE) ff_add(dh, dl, m * hv.x, m * hv.y);
    if (ds2 != 0) ff_add(dh, dl, (float)ds2 * Dv.x, (float)ds2 * Dv.y);
}

// The reference's FP64 rule for one Blume-Capel site (taken when the FP32 test cannot decide).
template <int ALG, bool EDGEJ, int FIELD>
__device__ __noinline__ int bc_exact_site(const GraphDev& g, const int8_t* sp, long long p, long long off, int w,
                                          int lane, int so, int isum, unsigned long long ku, uint32_t lo,
                                          double* dE_out) {
    double c = g.J * (double)isum;
    if (EDGEJ) {
        c = 0.0;
        for (int k = 0; k < w; ++k) {
            const long long e = off + 32ll * k + lane;
            const int nb = g.nbr[e];
            if (nb >= 0) c += g.J64[e] * (double)sp[nb];
        }
    }
    const double hf = FIELD == F_VECTOR ? g.h[p] : (FIELD == F_UNIFORM ? g.hu : 0.0);
    const double u = (double)ku * 0x1p-53;
    int sn;
    if (ALG == MCX_HEATBATH) {  // spin_flip!(::AbstractBlumeCapel, ::AbstractHeatBath), :61-85
        const double e1 = (c - hf * (-1.0)) + g.D;
        const double e3 = (-c - hf) + g.D;
        const double w1 = mcx_exp(-g.beta * e1), w2 = mcx_exp(-g.beta * 0.0), w3 = mcx_exp(-g.beta * e3);
        const double z = (w1 + w2) + w3;
        const double r = u * z;
        sn = r < w1 ? -1 : (r < w1 + w2 ? 0 : 1);
    } else {
        const int prop = bc_propose_state(so, (int)(lo & 1u));
        const double lr = -g.beta * bc_delta(c, so, prop, hf, FIELD != F_NONE, g.D);
        const bool acc = ALG == MCX_METROPOLIS ? ((lr > 0) || (u < mcx_exp(lr))) : (u < mcx_logistic(lr));
        sn = acc ? prop : so;
    }
    *dE_out = sn != so ? bc_delta(c, so, sn, hf, FIELD != F_NONE, g.D) : 0.0;
    return sn;
}

// One Blume-Capel site on the FP32 path: ΔE and the Boltzmann weights from the
// float-float coupling sum with proven error bounds (as for the Ising graphs), the
// decision certified against the FP64 rule, the exact evaluation when it cannot be.
template <int ALG, bool EDGEJ, int FIELD>
__device__ __forceinline__ int bc_decide_fast(const GraphDev& g, const int8_t* sp, long long p, long long off, int w,
                                              int lane, int so, const BcRowFF& r, uint32_t hi, uint32_t lo, float& eh,
                                              float& el) {
    const float2 hv = FIELD == F_VECTOR ? g.h2[p] : (FIELD == F_UNIFORM ? g.h2u : make_float2(0.0f, 0.0f));
    const float hm = fabsf(hv.x), Dm = fabsf(g.D2u.x);
    const float wf = (float)(w + 1);
    const float errc = wf * wf * r.S * 0x1p-45f;  // float-float coupling sum vs exact, doubled
    int sn = -2;
    if (ALG == MCX_HEATBATH) {
        float e1h = r.ch, e1l = r.cl, e3h = -r.ch, e3l = -r.cl;
        if (FIELD != F_NONE) {
            ff_add(e1h, e1l, hv.x, hv.y);
            ff_add(e3h, e3l, -hv.x, -hv.y);
        }
        ff_add(e1h, e1l, g.D2u.x, g.D2u.y);
        ff_add(e3h, e3l, g.D2u.x, g.D2u.y);
        const float e1 = e1h + e1l, e3 = e3h + e3l;
        const float x1 = -g.beta32 * e1, x3 = -g.beta32 * e3;
        const float b = fabsf(g.beta32) * 1.01f;
        const float ex1 = b * ((2.0f * r.S + 2.0f * hm + Dm + fabsf(e1)) * 0x1p-20f + errc) + fabsf(x1) * 0x1p-21f;
        const float ex3 = b * ((2.0f * r.S + 2.0f * hm + Dm + fabsf(e3)) * 0x1p-20f + errc) + fabsf(x3) * 0x1p-21f;
        const float m = 1.01f * (ex1 + ex3) + (fabsf(x1) + fabsf(x3)) * 0x1p-21f + 0x1p-19f;
        if (m < 0x1p-8f) {
            const float M = fmaxf(x1, fmaxf(0.0f, x3));
            const float q1 = __expf(x1 - M), q2 = __expf(-M), q3 = __expf(x3 - M);
            const float z = (q1 + q2) + q3;
            const int c1 = certain_u(q1 / z, m, hi);
            if (c1 == 1) {
                sn = -1;
            } else if (c1 == 0) {
                const int c2 = certain_u((q1 + q2) / z, m, hi);
                sn = c2 == 1 ? 0 : (c2 == 0 ? 1 : -2);
            }
        }
    } else {
        const int prop = bc_propose_state(so, (int)(lo & 1u));
        const int ds = prop - so, ds2 = prop * prop - so * so;
        float dh, dl;
        bc_delta_ff<FIELD>(r, hv, g.D2u, ds, ds2, dh, dl);
        const float df = dh + dl;
        const float ad = fabsf((float)ds);
        const float errd = (ad * (2.0f * r.S + hm) + Dm + fabsf(df)) * 0x1p-20f + ad * errc;
        const float xf = -g.beta32 * df;
        const float errx = fabsf(g.beta32) * errd * 1.01f + fabsf(xf) * 0x1p-21f + 0x1p-126f;
        const int c = certain_below<ALG != MCX_METROPOLIS>(xf, errx, hi);
        if (c >= 0) sn = c == 1 ? prop : so;
    }
    if (sn != -2) {
        if (sn != so) {
            float dh, dl;
            bc_delta_ff<FIELD>(r, hv, g.D2u, sn - so, sn * sn - so * so, dh, dl);
            ff_add(eh, el, dh, dl);
        }
        return sn;
    }
    const unsigned long long ku = ((unsigned long long)hi << 21) | (unsigned long long)(lo >> 11);
    double dE;
    sn = bc_exact_site<ALG, EDGEJ, FIELD>(g, sp, p, off, w, lane, so, r.isum, ku, lo, &dE);
    if (sn != so) {
        const float h = __double2float_rn(dE);
        ff_add(eh, el, h, __double2float_rn(dE - (double)h));
    }
    return sn;
}

// One Blume-Capel site: returns the new state (the old one when nothing changes) and adds
// the ΔE of a change to (eh, el).
template <int ALG, bool TABLE, bool EDGEJ, int FIELD>
__device__ __forceinline__ int bc_decide(const GraphDev& g, long long p, int so, int isum, double cacc, uint32_t hi,
                                         uint32_t lo, float& eh, float& el) {
    const unsigned long long ku = ((unsigned long long)hi << 21) | (unsigned long long)(lo >> 11);
    if (TABLE) {
        const int width = 2 * g.dmax + 1, idx = isum + g.dmax;
        int sn;
        if (ALG == MCX_HEATBATH) {
            sn = ku < g.tab[2 * idx] ? -1 : (ku < g.tab[2 * idx + 1] ? 0 : 1);
            if (sn != so) {
                const float2 d = g.tabdE[((so + 1) * 3 + sn + 1) * width + idx];
                ff_add(eh, el, d.x, d.y);
            }
        } else {
            const int b = (int)(lo & 1u);
            const int e = ((so + 1) * 2 + b) * width + idx;
            sn = ku < g.tab[e] ? bc_propose_state(so, b) : so;
            if (sn != so) {
                const float2 d = g.tabdE[e];
                ff_add(eh, el, d.x, d.y);
            }
        }
        return sn;
    }
    const double c = EDGEJ ? cacc : g.J * (double)isum;
    const double hf = FIELD == F_VECTOR ? g.h[p] : (FIELD == F_UNIFORM ? g.hu : 0.0);
    const double u = (double)ku * 0x1p-53;
    int sn;
    if (ALG == MCX_HEATBATH) {  // spin_flip!(::AbstractBlumeCapel, ::AbstractHeatBath), :61-85
        const double e1 = (c - hf * (-1.0)) + g.D;
        const double e3 = (-c - hf) + g.D;
        const double w1 = mcx_exp(-g.beta * e1), w2 = mcx_exp(-g.beta * 0.0), w3 = mcx_exp(-g.beta * e3);
        const double z = (w1 + w2) + w3;
        const double r = u * z;
        sn = r < w1 ? -1 : (r < w1 + w2 ? 0 : 1);
    } else {
        const int prop = bc_propose_state(so, (int)(lo & 1u));
        const double lr = -g.beta * bc_delta(c, so, prop, hf, FIELD != F_NONE, g.D);
        const bool acc = ALG == MCX_METROPOLIS ? ((lr > 0) || (u < mcx_exp(lr))) : (u < mcx_logistic(lr));
        sn = acc ? prop : so;
    }
    if (sn != so) {
        const double dE = bc_delta(c, so, sn, hf, FIELD != F_NONE, g.D);
        const float h = __double2float_rn(dE);
        ff_add(eh, el, h, __double2float_rn(dE - (double)h));
    }
    return sn;
}

template <int ALG, bool TABLE, bool EDGEJ, int FIELD>
__device__ __forceinline__ void bc_class_pairs(const GraphDev& g, int8_t* sp, const GClass& c, long long first,
                                               long long stride, int lane, uint32_t k0, uint32_t k1, uint32_t stream,
                                               unsigned long long sweep, float& eh, float& el, long long& dM,
                                               long long& nacc) {
    const uint32_t w2 = ctr_word2(sweep, 0, P_GRAPH);
    const long long npairs = (c.nslices + 1) >> 1;
    for (long long j = first; j < npairs; j += stride) {
        const long long sA = c.slice0 + 2 * j;
        const bool hasB = 2 * j + 1 < c.nslices;
        const long long pA = sA * 32 + lane, pB = pA + 32;
        const long long lA = 64 * j + lane, lB = lA + 32;
        const long long offA = g.soff[sA], offB = g.soff[sA + 1];
        const int wA = (int)((offB - offA) >> 5);
        const int wB = hasB ? (int)((g.soff[sA + 2] - offB) >> 5) : 0;
        const int soA = sp[pA];
        const int soB = hasB ? (int)sp[pB] : 0;
        int snA = soA, snB = soB;
        if (TABLE) {
            int iA, iB;
            double cA, cB;
            bc_row<false>(g, sp, offA, wA, lane, iA, cA);
            bc_row<false>(g, sp, offB, wB, lane, iB, cB);
            const uint4 r = philox10(make_uint4((uint32_t)(c.blk0 + 32 * j + lane), (uint32_t)sweep, w2, stream), k0, k1);
            if (lA < c.count) snA = bc_decide<ALG, true, false, FIELD>(g, pA, soA, iA, cA, r.x, r.y, eh, el);
            if (lB < c.count) snB = bc_decide<ALG, true, false, FIELD>(g, pB, soB, iB, cB, r.z, r.w, eh, el);
        } else {
            BcRowFF rA, rB;
            bc_row_ff<EDGEJ>(g, sp, offA, wA, lane, rA);
            bc_row_ff<EDGEJ>(g, sp, offB, wB, lane, rB);
            const uint4 r = philox10(make_uint4((uint32_t)(c.blk0 + 32 * j + lane), (uint32_t)sweep, w2, stream), k0, k1);
            if (lA < c.count)
                snA = bc_decide_fast<ALG, EDGEJ, FIELD>(g, sp, pA, offA, wA, lane, soA, rA, r.x, r.y, eh, el);
            if (lB < c.count)
                snB = bc_decide_fast<ALG, EDGEJ, FIELD>(g, sp, pB, offB, wB, lane, soB, rB, r.z, r.w, eh, el);
        }
        if (snA != soA) {
            sp[pA] = (int8_t)snA;
            dM += snA - soA;
            ++nacc;
        }
        if (snB != soB) {
            sp[pB] = (int8_t)snB;
            dM += snB - soB;
            ++nacc;
        }
    }
}

template <int ALG, bool TABLE, bool EDGEJ, int FIELD>
__global__ void __launch_bounds__(kGraphBlock, TABLE ? 5 : 4) k_bcg_class(GraphDev g, GClass c, uint32_t k0, uint32_t k1,
                                                           uint32_t stream, unsigned long long sweep) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    pdl_trigger();
    pdl_wait();  // the previous class (or sweep) is complete
    float eh = 0.0f, el = 0.0f;
    long long dM = 0, nacc = 0;
    bc_class_pairs<ALG, TABLE, EDGEJ, FIELD>(g, g.spins, c, (long long)blockIdx.x * kSlicesPerBlock + warp,
                                             (long long)gridDim.x * kSlicesPerBlock, lane, k0, k1, stream, sweep, eh,
                                             el, dM, nacc);
    const double t = block_sum_f64((double)eh + (double)el);
    if (threadIdx.x == 0) g.part[c.part0 + blockIdx.x] = t;
    dM = warp_sum_i64(dM);
    nacc = warp_sum_i64(nacc);
    if (lane == 0) {
        if (dM) atomicAdd(reinterpret_cast<unsigned long long*>(g.M), (unsigned long long)dM);
        if (nacc) atomicAdd(g.acc, (unsigned long long)nacc);
    }
}

// every sweep of a call on a small Blume-Capel graph in one block (as k_graph_small)
template <int ALG, bool TABLE, bool EDGEJ, int FIELD>
__global__ void __launch_bounds__(512, 1) k_bcg_small(GraphDev g, const GClass* __restrict__ classes, int ncls,
                                                      uint32_t k0, uint32_t k1, uint32_t stream,
                                                      unsigned long long sweep0, long long nsweeps, double* Eser,
                                                      long long* Mser, int npad) {
    extern __shared__ int8_t s_spins[];
    __shared__ float red_f[2][32];
    __shared__ long long red_i[2][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (int)(blockDim.x >> 5);
    for (int p = threadIdx.x; p < npad; p += blockDim.x) s_spins[p] = g.spins[p];
    double E = 0.0;
    long long M = 0, acc = 0;
    if (threadIdx.x == 0) {
        E = *g.E;
        M = *g.M;
    }
    __syncthreads();
    for (long long t = 0; t < nsweeps; ++t) {
        float eh = 0.0f, el = 0.0f;
        long long dM = 0, nacc = 0;
        for (int k = 0; k < ncls; ++k) {
            bc_class_pairs<ALG, TABLE, EDGEJ, FIELD>(g, s_spins, classes[k], warp, nw, lane, k0, k1, stream,
                                                     sweep0 + (unsigned long long)t, eh, el, dM, nacc);
            __syncthreads();
        }
        warp_ff_sum(eh, el);
        dM = warp_sum_i64(dM);
        nacc = warp_sum_i64(nacc);
        if (lane == 0) {
            red_f[0][warp] = eh;
            red_f[1][warp] = el;
            red_i[0][warp] = dM;
            red_i[1][warp] = nacc;
        }
        __syncthreads();
        if (warp == 0) {
            float h = lane < nw ? red_f[0][lane] : 0.0f, l = lane < nw ? red_f[1][lane] : 0.0f;
            long long m = lane < nw ? red_i[0][lane] : 0, a = lane < nw ? red_i[1][lane] : 0;
            warp_ff_sum(h, l);
            m = warp_sum_i64(m);
            a = warp_sum_i64(a);
            if (lane == 0) {
                E = E + ((double)h + (double)l);
                M += m;
                acc += a;
                if (Eser) Eser[t] = E;
                if (Mser) Mser[t] = M;
            }
        }
        __syncthreads();
    }
    for (int p = threadIdx.x; p < npad; p += blockDim.x) g.spins[p] = s_spins[p];
    if (threadIdx.x == 0) {
        *g.E = E;
        *g.M = M;
        *g.acc = *g.acc + (unsigned long long)acc;
    }
}

// delta_energy(sys, i, s_new) (op 0) or modify! to s_new (op 1) at one position.
template <bool EDGEJ, int FIELD>
__global__ void k_bcg_site(GraphDev g, long long p, int sn, int op, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const long long s = p >> 5;
    const int lane = (int)(p & 31);
    const long long off = g.soff[s];
    const int w = (int)((g.soff[s + 1] - off) >> 5);
    const int so = g.spins[p];
    int isum;
    double c;
    bc_row<EDGEJ>(g, g.spins, off, w, lane, isum, c);
    if (!EDGEJ) c = g.J * (double)isum;
    const double hf = FIELD == F_VECTOR ? g.h[p] : (FIELD == F_UNIFORM ? g.hu : 0.0);
    const double dE = bc_delta(c, so, sn, hf, FIELD != F_NONE, g.D);
    *out = dE;
    if (op == 1 && sn != so) {
        g.spins[p] = (int8_t)sn;
        *g.E = *g.E + dE;
        *g.M = *g.M + (sn - so);
    }
}

// spin_flip!(sys, alg) at uniformly random sites, one attempt after another (the reference's
// own order: pick_site, SpinSystems/src/abstractions.jl:19, then the site's FP64 rule, the
// exact path of the sweeps).  Attempt a draws Philox(seed, (a lo, a hi, 5<<24, stream)):
// vertex ((w0<<32)|w1) mod n, u = u53(w2, w3); a Blume-Capel Metropolis / Glauber proposal is
// the top bit of word 0 of (a lo, a hi, 6<<24, stream).  Lanes draw 32 attempts at a time,
// lane 0 applies them in order and keeps E as a sequential FP64 sum.
template <bool EDGEJ, int FIELD, bool BC>
__global__ void k_graph_seq(GraphDev g, const int32_t* __restrict__ perm, long long n, int alg, uint32_t k0,
                            uint32_t k1, uint32_t stream, unsigned long long a0, long long nat,
                            unsigned long long* counts) {
    __shared__ long long s_p[32];
    __shared__ unsigned long long s_k[32];
    __shared__ uint32_t s_b[32];
    const int lane = threadIdx.x & 31;
    if (threadIdx.x >= 32) return;
    double E = *g.E;
    long long M = *g.M;
    unsigned long long acc = 0;
    for (long long base = 0; base < nat; base += 32) {
        const long long m = nat - base < 32 ? nat - base : 32;
        if (lane < m) {
            const unsigned long long a = a0 + (unsigned long long)(base + lane);
            const uint4 w = philox10(make_uint4((uint32_t)a, (uint32_t)(a >> 32), 5u << 24, stream), k0, k1);
            const long long v = (long long)((((unsigned long long)w.x << 32) | w.y) % (unsigned long long)n);
            s_p[lane] = perm[v];
            s_k[lane] = ((unsigned long long)w.z << 21) | (unsigned long long)(w.w >> 11);
            s_b[lane] = BC && alg != MCX_HEATBATH
                            ? philox10(make_uint4((uint32_t)a, (uint32_t)(a >> 32), 6u << 24, stream), k0, k1).x >> 31
                            : 0u;
        }
        __syncwarp();
        if (lane == 0) {
            for (int j = 0; j < (int)m; ++j) {
                const long long p = s_p[j];
                const long long sl = p >> 5;
                const int ln = (int)(p & 31);
                const long long off = g.soff[sl];
                const int w = (int)((g.soff[sl + 1] - off) >> 5);
                const int so = g.spins[p];
                int isum = 0;
                if (!EDGEJ)
                    for (int k = 0; k < w; ++k) {
                        const int nb = g.nbr[off + 32ll * k + ln];
                        if (nb >= 0) isum += g.spins[nb];
                    }
                double dE = 0.0;
                int sn = so;
                if (BC) {
                    if (alg == MCX_METROPOLIS)
                        sn = bc_exact_site<MCX_METROPOLIS, EDGEJ, FIELD>(g, g.spins, p, off, w, ln, so, isum, s_k[j],
                                                                         s_b[j], &dE);
                    else if (alg == MCX_GLAUBER)
                        sn = bc_exact_site<MCX_GLAUBER, EDGEJ, FIELD>(g, g.spins, p, off, w, ln, so, isum, s_k[j],
                                                                      s_b[j], &dE);
                    else
                        sn = bc_exact_site<MCX_HEATBATH, EDGEJ, FIELD>(g, g.spins, p, off, w, ln, so, isum, s_k[j],
                                                                       s_b[j], &dE);
                } else {
                    bool flip;
                    if (alg == MCX_METROPOLIS)
                        flip = exact_site<MCX_METROPOLIS, EDGEJ, FIELD>(g, g.spins, p, off, w, ln, so, so * isum,
                                                                        s_k[j], &dE);
                    else if (alg == MCX_GLAUBER)
                        flip = exact_site<MCX_GLAUBER, EDGEJ, FIELD>(g, g.spins, p, off, w, ln, so, so * isum, s_k[j],
                                                                     &dE);
                    else
                        flip = exact_site<MCX_HEATBATH, EDGEJ, FIELD>(g, g.spins, p, off, w, ln, so, so * isum,
                                                                      s_k[j], &dE);
                    if (flip) sn = -so;
                }
                if (sn != so) {
                    g.spins[p] = (int8_t)sn;
                    E = E + dE;
                    M += sn - so;
                    ++acc;
                }
            }
        }
        __syncwarp();
    }
    if (lane == 0) {
        *g.E = E;
        *g.M = M;
        counts[0] = (unsigned long long)nat;
        counts[1] = acc;
    }
}

template <bool EDGEJ, bool BC>
cudaError_t seq_launch(int field, cudaStream_t st, void** args) {
    const void* fn = field == F_VECTOR    ? reinterpret_cast<const void*>(&k_graph_seq<EDGEJ, F_VECTOR, BC>)
                     : field == F_UNIFORM ? reinterpret_cast<const void*>(&k_graph_seq<EDGEJ, F_UNIFORM, BC>)
                                          : reinterpret_cast<const void*>(&k_graph_seq<EDGEJ, F_NONE, BC>);
    return cudaLaunchKernel(fn, dim3(1), dim3(32), args, 0, st);
}

// E += Σ partials (fixed order); record the series entry of sweep t.
__global__ void __launch_bounds__(kGraphBlock) k_graph_finish(double* part, int nparts, double* E, const long long* M,
                                                              double* Eser, long long* Mser, long long t) {
    pdl_trigger();
    pdl_wait();  // every class of the sweep is complete
    double v = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) v += part[i];
    const double s = block_sum_f64(v);
    if (threadIdx.x == 0) {
        const double e = *E + s;
        *E = e;
        if (Eser) Eser[t] = e;
        if (Mser) Mser[t] = *M;
    }
}

// _full_energy / sum(spins): per block the FP64 pair and field sums, one int64 atomic for
// the integer pair sum and for M.
template <bool EDGEJ, int FIELD>
__global__ void __launch_bounds__(kGraphBlock) k_graph_recompute(GraphDev g, long long nslices, double* part2,
                                                                 long long* ilpi, long long* qsum) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double pacc = 0.0, facc = 0.0;
    long long lsum = 0, msum = 0, q = 0;
    for (long long s = (long long)blockIdx.x * kSlicesPerBlock + warp; s < nslices;
         s += (long long)gridDim.x * kSlicesPerBlock) {
        const long long p = s * 32 + lane;
        const long long off = g.soff[s];
        const int w = (int)((g.soff[s + 1] - off) >> 5);
        const int si = g.spins[p];
        double acc = 0.0;
        int lpi = 0;
        for (int k = 0; k < w; ++k) {
            const long long e = off + 32ll * k + lane;
            const int nb = g.nbr[e];
            if (nb >= 0) {
                const int sj = g.spins[nb];
                if (EDGEJ) {
                    const double Jk = g.J64[e];
                    const int pr = si * sj;
                    if (pr != 0) acc += pr > 0 ? Jk : -Jk;  // (s_i J) s_j; products with 0 add nothing
                } else {
                    lpi += si * sj;
                }
            }
        }
        pacc += acc;
        lsum += lpi;
        msum += si;
        q += si * si;
        if (FIELD == F_VECTOR && si != 0) facc += g.h[p] * (double)si;
    }
    const double pt = block_sum_f64(pacc);
    const double ft = block_sum_f64(facc);
    if (threadIdx.x == 0) {
        part2[2 * blockIdx.x] = pt;
        part2[2 * blockIdx.x + 1] = ft;
    }
    lsum = warp_sum_i64(lsum);
    msum = warp_sum_i64(msum);
    q = warp_sum_i64(q);
    if (lane == 0) {
        if (q) atomicAdd(reinterpret_cast<unsigned long long*>(qsum), (unsigned long long)q);
        if (lsum) atomicAdd(reinterpret_cast<unsigned long long*>(ilpi), (unsigned long long)lsum);
        if (msum) atomicAdd(reinterpret_cast<unsigned long long*>(g.M), (unsigned long long)msum);
    }
}

// pair = Σ lpi / 2 (FP64 for the per-entry couplings, J (Σ lpi / 2) for one J);
// E = -pair - field (+ D Σ s² for Blume-Capel).
__global__ void __launch_bounds__(kGraphBlock) k_graph_recompute_finish(const double* part2, int nparts,
                                                                        const long long* ilpi, const long long* qsum,
                                                                        int edgej, int field, int bc, double J,
                                                                        double hu, double D, const long long* M,
                                                                        double* E) {
    double p = 0.0, f = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        p += part2[2 * i];
        f += part2[2 * i + 1];
    }
    const double ps = block_sum_f64(p);
    const double fs = block_sum_f64(f);
    if (threadIdx.x == 0) {
        const double pair = edgej ? ps / 2 : J * (double)(*ilpi / 2);
        const double fld = field == F_VECTOR ? fs : field == F_UNIFORM ? hu * (double)(*M) : 0.0;
        const double e = field == F_NONE ? -pair : -pair - fld;
        *E = bc ? (-pair - fld) + D * (double)(*qsum) : e;
    }
}

// delta_energy(sys, i) (op 0) or modify! with flip_changes (op 1) at one position;
// target -1 / +1 is a state to move to (no change when it is the current one), 2 a flip.
template <bool EDGEJ, int FIELD>
__global__ void k_graph_site(GraphDev g, long long p, int target, int op, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const long long s = p >> 5;
    const int lane = (int)(p & 31);
    const long long off = g.soff[s];
    const int w = (int)((g.soff[s + 1] - off) >> 5);
    const int si = g.spins[p];
    if (target != 2 && target == si) {
        *out = 0.0;
        return;
    }
    int lpi = 0;
    if (!EDGEJ)
        for (int k = 0; k < w; ++k) {
            const int nb = g.nbr[off + 32ll * k + lane];
            if (nb >= 0) lpi += si * g.spins[nb];
        }
    const double dE = site_delta_energy<EDGEJ, FIELD>(g, g.spins, p, off, w, lane, si, lpi);
    *out = dE;
    if (op == 1) {
        g.spins[p] = (int8_t)(-si);
        *g.E = *g.E + dE;
        *g.M = *g.M - 2 * si;
    }
}

__global__ void k_graph_validate(const int8_t* lin, long long n, int bc, unsigned long long* bad) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const int8_t x = lin[v];
        if (x != 1 && x != -1 && !(bc && x == 0)) atomicAdd(bad, 1ull);
    }
}

__global__ void k_graph_scatter(const int8_t* lin, const int32_t* perm, long long n, int8_t* spins) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
        spins[perm[v]] = lin[v];
}

__global__ void k_graph_gather(int8_t* lin, const int32_t* perm, long long n, const int8_t* spins) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
        lin[v] = spins[perm[v]];
}

// init!(sys, :random): site v takes word v&3 of Philox block (v>>2, 0, P_GRAPH_INIT<<24,
// stream): its top bit (Ising, +1 / -1) or floor(3 w / 2^32) - 1 (Blume-Capel).
__global__ void k_graph_init_random(const int32_t* perm, long long n, int8_t* spins, uint32_t k0, uint32_t k1,
                                    uint32_t stream, int bc) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const uint4 r = philox10(make_uint4((uint32_t)(v >> 2), 0u, (uint32_t)P_GRAPH_INIT << 24, stream), k0, k1);
        const uint32_t wv = pick4(r, (int)(v & 3));
        spins[perm[v]] = bc ? (int8_t)((int)(((unsigned long long)wv * 3ull) >> 32) - 1) : ((wv & 0x80000000u) ? 1 : -1);
    }
}

__global__ void k_graph_init_uniform(const int32_t* perm, long long n, int8_t* spins, int8_t value) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
        spins[perm[v]] = value;
}

using ClassFn = void (*)(GraphDev, GClass, uint32_t, uint32_t, uint32_t, unsigned long long);
using SmallFn = void (*)(GraphDev, const GClass*, int, uint32_t, uint32_t, uint32_t, unsigned long long, long long,
                         double*, long long*, int);

struct SweepFns {
    ClassFn cls;        // one class per launch
    SmallFn small;      // all sweeps in one block
    int small_threads;  // its block size
};

template <int ALG, bool TABLE, bool EDGEJ, int FIELD>
SweepFns fns_of() {
    return {k_graph_class<ALG, TABLE, EDGEJ, FIELD>, k_graph_small<ALG, TABLE, EDGEJ, FIELD>, small_block(TABLE)};
}

template <int ALG, bool TABLE>
SweepFns sweep_fns_t(bool edgej, int field) {
    if (TABLE) return field == F_UNIFORM ? fns_of<ALG, true, false, F_UNIFORM>() : fns_of<ALG, true, false, F_NONE>();
    if (edgej)
        return field == F_VECTOR    ? fns_of<ALG, false, true, F_VECTOR>()
               : field == F_UNIFORM ? fns_of<ALG, false, true, F_UNIFORM>()
                                    : fns_of<ALG, false, true, F_NONE>();
    return field == F_VECTOR    ? fns_of<ALG, false, false, F_VECTOR>()
           : field == F_UNIFORM ? fns_of<ALG, false, false, F_UNIFORM>()
                                : fns_of<ALG, false, false, F_NONE>();
}

template <int ALG, bool TABLE, bool EDGEJ, int FIELD>
SweepFns bc_fns_of() {
    return {k_bcg_class<ALG, TABLE, EDGEJ, FIELD>, k_bcg_small<ALG, TABLE, EDGEJ, FIELD>, 512};
}

template <int ALG, bool TABLE>
SweepFns bc_sweep_fns_t(bool edgej, int field) {
    if (TABLE) return field == F_UNIFORM ? bc_fns_of<ALG, true, false, F_UNIFORM>() : bc_fns_of<ALG, true, false, F_NONE>();
    if (edgej)
        return field == F_VECTOR    ? bc_fns_of<ALG, false, true, F_VECTOR>()
               : field == F_UNIFORM ? bc_fns_of<ALG, false, true, F_UNIFORM>()
                                    : bc_fns_of<ALG, false, true, F_NONE>();
    return field == F_VECTOR    ? bc_fns_of<ALG, false, false, F_VECTOR>()
           : field == F_UNIFORM ? bc_fns_of<ALG, false, false, F_UNIFORM>()
                                : bc_fns_of<ALG, false, false, F_NONE>();
}

SweepFns bc_sweep_fns(mcx_algorithm alg, bool table, bool edgej, int field) {
    switch (alg) {
        case MCX_METROPOLIS: return table ? bc_sweep_fns_t<MCX_METROPOLIS, true>(edgej, field)
                                          : bc_sweep_fns_t<MCX_METROPOLIS, false>(edgej, field);
        case MCX_GLAUBER: return table ? bc_sweep_fns_t<MCX_GLAUBER, true>(edgej, field)
                                       : bc_sweep_fns_t<MCX_GLAUBER, false>(edgej, field);
        default: return table ? bc_sweep_fns_t<MCX_HEATBATH, true>(edgej, field)
                              : bc_sweep_fns_t<MCX_HEATBATH, false>(edgej, field);
    }
}

SweepFns sweep_fns(mcx_algorithm alg, bool table, bool edgej, int field) {
    switch (alg) {
        case MCX_METROPOLIS: return table ? sweep_fns_t<MCX_METROPOLIS, true>(edgej, field)
                                          : sweep_fns_t<MCX_METROPOLIS, false>(edgej, field);
        case MCX_GLAUBER: return table ? sweep_fns_t<MCX_GLAUBER, true>(edgej, field)
                                       : sweep_fns_t<MCX_GLAUBER, false>(edgej, field);
        default: return table ? sweep_fns_t<MCX_HEATBATH, true>(edgej, field)
                              : sweep_fns_t<MCX_HEATBATH, false>(edgej, field);
    }
}

template <bool EDGEJ>
void recompute_launch(int field, int grid, cudaStream_t st, const GraphDev& g, long long nslices, double* part2,
                      long long* ilpi, long long* qsum) {
    if (field == F_VECTOR)
        k_graph_recompute<EDGEJ, F_VECTOR><<<grid, kGraphBlock, 0, st>>>(g, nslices, part2, ilpi, qsum);
    else if (field == F_UNIFORM)
        k_graph_recompute<EDGEJ, F_UNIFORM><<<grid, kGraphBlock, 0, st>>>(g, nslices, part2, ilpi, qsum);
    else k_graph_recompute<EDGEJ, F_NONE><<<grid, kGraphBlock, 0, st>>>(g, nslices, part2, ilpi, qsum);
}

template <bool EDGEJ>
void site_launch(bool bc, int field, cudaStream_t st, const GraphDev& g, long long p, int target, int op,
                 double* out) {
    if (bc) {
        if (field == F_VECTOR) k_bcg_site<EDGEJ, F_VECTOR><<<1, 32, 0, st>>>(g, p, target, op, out);
        else if (field == F_UNIFORM) k_bcg_site<EDGEJ, F_UNIFORM><<<1, 32, 0, st>>>(g, p, target, op, out);
        else k_bcg_site<EDGEJ, F_NONE><<<1, 32, 0, st>>>(g, p, target, op, out);
        return;
    }
    if (field == F_VECTOR) k_graph_site<EDGEJ, F_VECTOR><<<1, 32, 0, st>>>(g, p, target, op, out);
    else if (field == F_UNIFORM) k_graph_site<EDGEJ, F_UNIFORM><<<1, 32, 0, st>>>(g, p, target, op, out);
    else k_graph_site<EDGEJ, F_NONE><<<1, 32, 0, st>>>(g, p, target, op, out);
}

// 53-bit threshold of "u < p" for u = k 2^-53: k < ceil(p 2^53).
// x = hi + lo with hi = fl32(x), lo = fl32(x - hi)
float2 split2(double x) {
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

unsigned long long threshold53(double p) {
    if (!(p > 0.0)) return 0;
    if (p >= 1.0) return 1ull << 53;
    return (unsigned long long)std::ceil(p * 9007199254740992.0);
}

}  // namespace

struct mcx_graph {
    mcx_ctx* ctx = nullptr;
    mcx::CtxHold hold;
    int64_t n = 0, npad = 0, nslices = 0, entries = 0;
    int ncol = 0;
    int dmax = 0;
    bool edgej = false;
    int field = F_NONE;
    bool bc = false;                // Blume-Capel (spins in {-1, 0, 1})
    double J = 1.0, h = 0.0, D = 0.0;
    std::vector<int32_t> colour;    // per vertex
    std::vector<GClass> classes;
    int nparts = 0;                 // partial-sum slots over all classes
    int8_t* d_spins = nullptr;
    int32_t* d_nbr = nullptr;
    double* d_J64 = nullptr;
    float2* d_J2 = nullptr;
    float2* d_h2 = nullptr;
    long long* d_soff = nullptr;
    double* d_h = nullptr;
    int32_t* d_perm = nullptr;      // vertex -> padded position
    int8_t* d_lin = nullptr;        // staging, vertex order
    unsigned long long* d_tab = nullptr;
    float2* d_tabdE = nullptr;
    int tab_alg = -1;
    double tab_beta = 0.0;
    double* d_E = nullptr;
    long long* d_M = nullptr;
    unsigned long long* d_acc = nullptr;
    long long* d_ilpi = nullptr;
    long long* d_qsum = nullptr;
    double* d_part = nullptr;
    int part_cap = 0;               // doubles
    double* d_Eser = nullptr;
    long long* d_Mser = nullptr;
    int64_t ser_cap = 0;
    int64_t ser_len = 0;            // sweeps recorded by the last sweep call
    double* d_site = nullptr;       // delta_energy result
    GClass* d_classes = nullptr;    // the class descriptors (one-block kernel)
    int64_t device_bytes = 0;
    std::vector<std::pair<void*, size_t>> allocs;

    bool table_mode() const { return !edgej && field != F_VECTOR && dmax <= kMaxTableDegree; }
    GraphDev dev(double beta) const {
        GraphDev g;
        g.spins = d_spins;
        g.nbr = d_nbr;
        g.J64 = d_J64;
        g.J2 = d_J2;
        g.h2 = d_h2;
        g.J2u = split2(J);
        g.h2u = split2(h);
        g.D2u = split2(D);
        g.beta32 = (float)beta;
        g.D = D;
        g.soff = d_soff;
        g.h = d_h;
        g.J = J;
        g.hu = h;
        g.tab = d_tab;
        g.tabdE = d_tabdE;
        g.dmax = dmax;
        g.beta = beta;
        g.acc = d_acc;
        g.M = d_M;
        g.E = d_E;
        g.part = d_part;
        return g;
    }
};

namespace {

template <typename T>
mcx_status galloc(mcx_graph* g, T** p, size_t count) {
    void* q = nullptr;
    MCX_CHECK(dev_alloc(g->ctx, &q, count * sizeof(T)));
    g->allocs.push_back({q, count * sizeof(T)});
    g->device_bytes += (int64_t)(count * sizeof(T));
    *p = static_cast<T*>(q);
    return MCX_OK;
}

void gfree(mcx_graph* g, void* p) {
    for (size_t i = 0; i < g->allocs.size(); ++i)
        if (g->allocs[i].first == p) {
            dev_free(g->ctx, p, g->allocs[i].second);
            g->device_bytes -= (int64_t)g->allocs[i].second;
            g->allocs.erase(g->allocs.begin() + (long)i);
            return;
        }
}

int grid_of(const mcx_graph* g, long long slices, int per_sm = 8) {
    long long b = (slices + kSlicesPerBlock - 1) / kSlicesPerBlock;
    long long cap = (long long)g->ctx->num_sms * per_sm;
    return (int)std::max(1ll, std::min(b, cap));
}

mcx_status graph_recompute(mcx_graph* g) {
    cudaStream_t st = g->ctx->stream;
    const int grid = grid_of(g, g->nslices);
    if (2 * grid > g->part_cap) return fail(MCX_ERR_INVALID_ARG, "partial-sum buffer too small");
    MCX_CUDA(cudaMemsetAsync(g->d_M, 0, sizeof(long long), st));
    MCX_CUDA(cudaMemsetAsync(g->d_ilpi, 0, sizeof(long long), st));
    MCX_CUDA(cudaMemsetAsync(g->d_qsum, 0, sizeof(long long), st));
    const GraphDev d = g->dev(0.0);
    if (g->edgej) recompute_launch<true>(g->field, grid, st, d, g->nslices, g->d_part, g->d_ilpi, g->d_qsum);
    else recompute_launch<false>(g->field, grid, st, d, g->nslices, g->d_part, g->d_ilpi, g->d_qsum);
    k_graph_recompute_finish<<<1, kGraphBlock, 0, st>>>(g->d_part, grid, g->d_ilpi, g->d_qsum, g->edgej ? 1 : 0,
                                                        g->field, g->bc ? 1 : 0, g->J, g->h, g->D, g->d_M, g->d_E);
    count_launch(g->ctx, 2);
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

// smallest k in [0, 2^53] with fl(fl(k 2^-53) z) >= w: "r = u z < w" holds exactly for k below
// it (fl(u z) does not decrease as u grows)
unsigned long long bisect53(double z, double w) {
    unsigned long long lo = 0, hi = 1ull << 53;
    while (lo < hi) {
        const unsigned long long mid = lo + (hi - lo) / 2;
        if (((double)mid * 0x1p-53) * z < w) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Blume-Capel tables by the neighbour sum: Metropolis / Glauber [(s_old+1)*2 + b][sum]
// thresholds and ΔE; heat bath [sum] (T1, T2) and ΔE by [(s_old+1)*3 + s_new+1][sum].
mcx_status bc_graph_table(mcx_graph* g, mcx_algorithm alg, double beta) {
    const int D_ = g->dmax, width = 2 * D_ + 1;
    const bool fld = g->field != F_NONE;
    const double hf = fld ? g->h : 0.0;
    std::vector<unsigned long long> thr(6 * (size_t)width, 0);
    std::vector<float2> dE(9 * (size_t)width, make_float2(0.0f, 0.0f));
    for (int sum = -D_; sum <= D_; ++sum) {
        const int idx = sum + D_;
        const double c = g->J * (double)sum;
        if (alg == MCX_HEATBATH) {
            const double e1 = (c - hf * (-1.0)) + g->D;
            const double e3 = (-c - hf) + g->D;
            const double w1 = mcx_exp(-beta * e1), w2 = mcx_exp(-beta * 0.0), w3 = mcx_exp(-beta * e3);
            const double z = (w1 + w2) + w3;
            thr[2 * (size_t)idx] = bisect53(z, w1);
            thr[2 * (size_t)idx + 1] = bisect53(z, w1 + w2);
            for (int so = -1; so <= 1; ++so)
                for (int sn = -1; sn <= 1; ++sn)
                    dE[(size_t)((so + 1) * 3 + sn + 1) * width + idx] = split2(bc_delta(c, so, sn, hf, fld, g->D));
        } else {
            for (int so = -1; so <= 1; ++so)
                for (int b = 0; b < 2; ++b) {
                    const int sn = bc_propose_state(so, b);
                    const double de = bc_delta(c, so, sn, hf, fld, g->D);
                    const double lr = -beta * de;
                    const size_t e = (size_t)((so + 1) * 2 + b) * width + idx;
                    thr[e] = alg == MCX_METROPOLIS ? (lr > 0 ? kAlways53 : threshold53(mcx_exp(lr)))
                                                   : threshold53(mcx_logistic(lr));
                    dE[e] = split2(de);
                }
        }
    }
    MCX_CUDA(cudaMemcpyAsync(g->d_tab, thr.data(), thr.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                             g->ctx->stream));
    MCX_CUDA(cudaMemcpyAsync(g->d_tabdE, dE.data(), dE.size() * sizeof(float2), cudaMemcpyHostToDevice,
                             g->ctx->stream));
    MCX_CUDA(cudaStreamSynchronize(g->ctx->stream));
    g->tab_alg = (int)alg;
    g->tab_beta = beta;
    return MCX_OK;
}

mcx_status graph_table(mcx_graph* g, mcx_algorithm alg, double beta) {
    if (g->tab_alg == (int)alg && g->tab_beta == beta) return MCX_OK;
    if (g->bc) return bc_graph_table(g, alg, beta);
    const int D = g->dmax, width = 2 * D + 1;
    std::vector<unsigned long long> thr(2 * (size_t)width);
    std::vector<float2> dE(2 * (size_t)width);
    for (int sp = 0; sp < 2; ++sp) {
        const int s = sp ? 1 : -1;
        for (int lpi = -D; lpi <= D; ++lpi) {
            const double dpair = (-2.0 * g->J) * (double)lpi;
            const double dspin = (double)(-2 * s);
            const double de = g->field == F_UNIFORM ? -dpair - g->h * dspin : -dpair;
            unsigned long long t;
            if (alg == MCX_METROPOLIS) {
                const double lr = -beta * de;
                t = lr > 0 ? kAlways53 : threshold53(mcx_exp(lr));
            } else if (alg == MCX_GLAUBER) {
                t = threshold53(mcx_logistic(-beta * de));
            } else {
                t = threshold53(mcx_logistic((beta * (double)s) * de));
            }
            thr[(size_t)sp * width + (lpi + D)] = t;
            dE[(size_t)sp * width + (lpi + D)] = split2(de);
        }
    }
    MCX_CUDA(cudaMemcpyAsync(g->d_tab, thr.data(), thr.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                             g->ctx->stream));
    MCX_CUDA(cudaMemcpyAsync(g->d_tabdE, dE.data(), dE.size() * sizeof(float2), cudaMemcpyHostToDevice,
                             g->ctx->stream));
    // the host vectors go out of scope: wait for the copies
    MCX_CUDA(cudaStreamSynchronize(g->ctx->stream));
    g->tab_alg = (int)alg;
    g->tab_beta = beta;
    return MCX_OK;
}

}  // namespace

extern "C" {

static mcx_status graph_create(mcx_ctx* ctx, bool bc, int64_t n, const int64_t* rowptr, const int32_t* col,
                               const double* coupling, double J, double D, const double* field, double h,
                               mcx_graph** out) {
    if (!ctx || !rowptr || !out || (!col && n > 0)) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (n < 1 || n > (1ll << 30)) return fail(MCX_ERR_INVALID_ARG, "n = %lld sites (1 .. 2^30)", (long long)n);
    if (rowptr[0] != 0) return fail(MCX_ERR_INVALID_ARG, "rowptr[0] must be 0");
    for (int64_t v = 0; v < n; ++v)
        if (rowptr[v + 1] < rowptr[v]) return fail(MCX_ERR_INVALID_ARG, "rowptr decreases at %lld", (long long)v);
    if (!std::isfinite(J) || !std::isfinite(h) || !std::isfinite(D))
        return fail(MCX_ERR_INVALID_ARG, "J, D and h must be finite");
    // neighbour lists: in range, strictly increasing; symmetric with equal couplings
    std::vector<int32_t> deg(n, 0);
    for (int64_t v = 0; v < n; ++v) {
        for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e) {
            const int32_t u = col[e];
            if (u < 0 || u >= n) return fail(MCX_ERR_INVALID_ARG, "neighbour %d of site %lld out of range", u, (long long)v);
            if (e > rowptr[v] && col[e - 1] >= u)
                return fail(MCX_ERR_INVALID_ARG, "neighbours of site %lld are not strictly increasing", (long long)v);
            if (coupling && !std::isfinite(coupling[e])) return fail(MCX_ERR_INVALID_ARG, "coupling not finite");
            if (u == v) continue;
            ++deg[v];
            const int32_t* b = col + rowptr[u];
            const int32_t* en = col + rowptr[u + 1];
            const int32_t* f = std::lower_bound(b, en, (int32_t)v);
            if (f == en || *f != v) return fail(MCX_ERR_INVALID_ARG, "J must be symmetric: (%lld, %d) has no (%d, %lld)",
                                                (long long)v, u, u, (long long)v);
            if (coupling && coupling[e] != coupling[rowptr[u] + (f - b)])
                return fail(MCX_ERR_INVALID_ARG, "J must be symmetric: J[%lld,%d] != J[%d,%lld]", (long long)v, u, u,
                            (long long)v);
        }
    }
    if (field)
        for (int64_t v = 0; v < n; ++v)
            if (!std::isfinite(field[v])) return fail(MCX_ERR_INVALID_ARG, "field not finite");
    auto g = new mcx_graph();
    g->ctx = ctx;
    g->hold.set(ctx);
    g->n = n;
    g->edgej = coupling != nullptr;
    g->field = field ? F_VECTOR : (h != 0.0 ? F_UNIFORM : F_NONE);
    g->J = J;
    g->h = h;
    g->bc = bc;
    g->D = D;
    int dmax = 0;
    for (int64_t v = 0; v < n; ++v) dmax = std::max(dmax, deg[v]);
    g->dmax = dmax;
    // first-fit colouring in vertex order
    g->colour.assign(n, 0);
    std::vector<int64_t> seen((size_t)dmax + 2, -1);
    int ncol = 0;
    for (int64_t v = 0; v < n; ++v) {
        for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e)
            if (col[e] < v) seen[g->colour[col[e]]] = v;
        int c = 0;
        while (seen[c] == v) ++c;
        g->colour[v] = c;
        ncol = std::max(ncol, c + 1);
    }
    g->ncol = ncol;
    // renumbering: classes in turn, vertex order inside, each class padded to 32
    std::vector<int64_t> count(ncol, 0);
    for (int64_t v = 0; v < n; ++v) ++count[g->colour[v]];
    std::vector<int64_t> start(ncol + 1, 0);
    for (int c = 0; c < ncol; ++c) start[c + 1] = start[c] + (count[c] + 31) / 32 * 32;
    g->npad = start[ncol];
    g->nslices = g->npad / 32;
    if (g->npad >= (1ll << 31)) {
        delete g;
        return fail(MCX_ERR_INVALID_ARG, "graph too large");
    }
    std::vector<int32_t> perm(n);
    std::vector<int64_t> vert(g->npad, -1);  // position -> vertex
    {
        std::vector<int64_t> fill(start.begin(), start.end() - 1);
        for (int64_t v = 0; v < n; ++v) {
            const int64_t p = fill[g->colour[v]]++;
            perm[v] = (int32_t)p;
            vert[p] = v;
        }
    }
    int64_t blk0 = 0;
    int part0 = 0;
    const long long cap_blocks = (long long)ctx->num_sms * 8;
    for (int c = 0; c < ncol; ++c) {
        GClass k;
        k.p0 = start[c];
        k.count = count[c];
        k.blk0 = blk0;
        k.slice0 = start[c] / 32;
        k.nslices = (start[c + 1] - start[c]) / 32;
        k.part0 = part0;
        blk0 += 32 * ((k.nslices + 1) / 2);
        part0 += (int)std::min((k.nslices + kSlicesPerBlock - 1) / kSlicesPerBlock, cap_blocks);
        g->classes.push_back(k);
    }
    g->nparts = part0;
    // sliced-ELL entries
    std::vector<long long> soff(g->nslices + 1, 0);
    for (int64_t s = 0; s < g->nslices; ++s) {
        int w = 0;
        for (int l = 0; l < 32; ++l) {
            const int64_t v = vert[s * 32 + l];
            if (v >= 0) w = std::max(w, deg[v]);
        }
        soff[s + 1] = soff[s] + 32ll * w;
    }
    g->entries = soff[g->nslices];
    std::vector<int32_t> nbr(g->entries, -1);
    std::vector<double> jv(g->edgej ? g->entries : 0, 0.0);
    for (int64_t s = 0; s < g->nslices; ++s)
        for (int l = 0; l < 32; ++l) {
            const int64_t v = vert[s * 32 + l];
            if (v < 0) continue;
            int k = 0;
            for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e) {
                if (col[e] == v) continue;
                const int64_t idx = soff[s] + 32ll * k + l;
                nbr[idx] = perm[col[e]];
                if (g->edgej) jv[idx] = coupling[e];
                ++k;
            }
        }
    std::vector<double> hv;
    std::vector<float2> hv2;
    if (field) {
        hv.assign(g->npad, 0.0);
        for (int64_t v = 0; v < n; ++v) hv[perm[v]] = field[v];
        hv2.resize(g->npad);
        for (int64_t p = 0; p < g->npad; ++p) hv2[p] = split2(hv[p]);
    }
    std::vector<float2> jv2(jv.size());
    for (size_t k = 0; k < jv.size(); ++k) jv2[k] = split2(jv[k]);
    // device arrays
    mcx_status st = MCX_OK;
    const size_t tabn = (bc ? 6 : 2) * (size_t)(2 * dmax + 1), tabdn = (bc ? 9 : 2) * (size_t)(2 * dmax + 1);
    g->part_cap = std::max(g->nparts, 2 * (int)cap_blocks);
    do {
        if ((st = galloc(g, &g->d_spins, (size_t)g->npad))) break;
        if ((st = galloc(g, &g->d_nbr, (size_t)std::max<int64_t>(g->entries, 1)))) break;
        if (g->edgej && (st = galloc(g, &g->d_J64, (size_t)std::max<int64_t>(g->entries, 1)))) break;
        if (g->edgej && (st = galloc(g, &g->d_J2, (size_t)std::max<int64_t>(g->entries, 1)))) break;
        if ((st = galloc(g, &g->d_soff, (size_t)g->nslices + 1))) break;
        if (field && (st = galloc(g, &g->d_h, (size_t)g->npad))) break;
        if (field && (st = galloc(g, &g->d_h2, (size_t)g->npad))) break;
        if ((st = galloc(g, &g->d_perm, (size_t)n))) break;
        if ((st = galloc(g, &g->d_lin, (size_t)n))) break;
        if (g->table_mode() && (st = galloc(g, &g->d_tab, tabn))) break;
        if (g->table_mode() && (st = galloc(g, &g->d_tabdE, tabdn))) break;
        if ((st = galloc(g, &g->d_E, 1))) break;
        if ((st = galloc(g, &g->d_M, 1))) break;
        if ((st = galloc(g, &g->d_acc, 1))) break;
        if ((st = galloc(g, &g->d_ilpi, 1))) break;
        if ((st = galloc(g, &g->d_qsum, 1))) break;
        if ((st = galloc(g, &g->d_site, 1))) break;
        if ((st = galloc(g, &g->d_classes, (size_t)ncol))) break;
        if ((st = galloc(g, &g->d_part, (size_t)g->part_cap))) break;
    } while (false);
    if (st != MCX_OK) {
        mcx_graph_destroy(g);
        return st;
    }
    cudaStream_t s0 = ctx->stream;
    // every host vector outlives the copies: synchronize before returning
    std::vector<int8_t> spins(g->npad, 0);
    for (int64_t v = 0; v < n; ++v) spins[perm[v]] = 1;
    cudaError_t e = cudaSuccess;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s0);
    };
    up(g->d_spins, spins.data(), spins.size());
    up(g->d_nbr, nbr.data(), nbr.size() * sizeof(int32_t));
    if (g->edgej) up(g->d_J64, jv.data(), jv.size() * sizeof(double));
    if (g->edgej) up(g->d_J2, jv2.data(), jv2.size() * sizeof(float2));
    up(g->d_soff, soff.data(), soff.size() * sizeof(long long));
    if (field) up(g->d_h, hv.data(), hv.size() * sizeof(double));
    if (field) up(g->d_h2, hv2.data(), hv2.size() * sizeof(float2));
    up(g->d_perm, perm.data(), perm.size() * sizeof(int32_t));
    up(g->d_classes, g->classes.data(), g->classes.size() * sizeof(GClass));
    if (e == cudaSuccess) e = cudaMemsetAsync(g->d_acc, 0, sizeof(unsigned long long), s0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s0);
    if (e != cudaSuccess) {
        mcx_graph_destroy(g);
        return cuda_fail(e, "graph upload");
    }
    if ((st = graph_recompute(g)) != MCX_OK) {
        mcx_graph_destroy(g);
        return st;
    }
    *out = g;
    return MCX_OK;
}

MCX_API mcx_status mcx_graph_create(mcx_ctx* ctx, int64_t n, const int64_t* rowptr, const int32_t* col,
                                    const double* coupling, double J, const double* field, double h,
                                    mcx_graph** out) {
    return graph_create(ctx, false, n, rowptr, col, coupling, J, 0.0, field, h, out);
}

MCX_API mcx_status mcx_bcgraph_create(mcx_ctx* ctx, int64_t n, const int64_t* rowptr, const int32_t* col,
                                      const double* coupling, double J, double D, const double* field, double h,
                                      mcx_graph** out) {
    return graph_create(ctx, true, n, rowptr, col, coupling, J, D, field, h, out);
}

MCX_API mcx_status mcx_graph_destroy(mcx_graph* g) {
    if (!g) return MCX_OK;
    if (g->ctx) cudaStreamSynchronize(g->ctx->stream);
    while (!g->allocs.empty()) gfree(g, g->allocs.back().first);
    delete g;
    return MCX_OK;
}

MCX_API mcx_status mcx_graph_info(const mcx_graph* g, int64_t* nsites, int32_t* colours, int64_t* entries,
                                  int64_t* device_bytes) {
    if (!g) return fail(MCX_ERR_INVALID_ARG, "graph is NULL");
    if (nsites) *nsites = g->n;
    if (colours) *colours = g->ncol;
    if (entries) *entries = g->entries;
    if (device_bytes) *device_bytes = g->device_bytes;
    return MCX_OK;
}

MCX_API mcx_status mcx_graph_colours(const mcx_graph* g, int32_t* colour, size_t n) {
    if (!g || !colour) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if ((int64_t)n != g->n) return fail(MCX_ERR_INVALID_ARG, "expected %lld sites, got %zu", (long long)g->n, n);
    std::copy(g->colour.begin(), g->colour.end(), colour);
    return MCX_OK;
}

MCX_API mcx_status mcx_graph_set_spins(mcx_graph* g, const int8_t* host, size_t n) {
    if (!g || !host) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if ((int64_t)n != g->n) return fail(MCX_ERR_INVALID_ARG, "expected %lld spins, got %zu", (long long)g->n, n);
    cudaStream_t st = g->ctx->stream;
    MCX_CUDA(cudaMemcpyAsync(g->d_lin, host, n, cudaMemcpyHostToDevice, st));
    MCX_CUDA(cudaMemsetAsync(g->d_acc, 0, sizeof(unsigned long long), st));
    // values are checked on the device before any is stored (the counter word is free here)
    unsigned long long bad = 0;
    const int grid = (int)std::min<long long>((g->n + 255) / 256, (long long)g->ctx->num_sms * 8);
    k_graph_validate<<<grid, 256, 0, st>>>(g->d_lin, g->n, g->bc ? 1 : 0, g->d_acc);
    count_launch(g->ctx);
    MCX_CUDA(cudaGetLastError());
    MCX_CUDA(cudaMemcpyAsync(&bad, g->d_acc, sizeof(bad), cudaMemcpyDeviceToHost, st));
    MCX_CUDA(cudaStreamSynchronize(st));
    if (bad) return fail(MCX_ERR_INVALID_ARG, "%llu values are not spin states of this model", bad);
    k_graph_scatter<<<grid, 256, 0, st>>>(g->d_lin, g->d_perm, g->n, g->d_spins);
    count_launch(g->ctx);
    MCX_CUDA(cudaGetLastError());
    return graph_recompute(g);
}

MCX_API mcx_status mcx_graph_get_spins(mcx_graph* g, int8_t* host, size_t n) {
    if (!g || !host) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if ((int64_t)n != g->n) return fail(MCX_ERR_INVALID_ARG, "expected %lld spins, got %zu", (long long)g->n, n);
    cudaStream_t st = g->ctx->stream;
    const int grid = (int)std::min<long long>((g->n + 255) / 256, (long long)g->ctx->num_sms * 8);
    k_graph_gather<<<grid, 256, 0, st>>>(g->d_lin, g->d_perm, g->n, g->d_spins);
    count_launch(g->ctx);
    MCX_CUDA(cudaGetLastError());
    MCX_CUDA(cudaMemcpyAsync(host, g->d_lin, n, cudaMemcpyDeviceToHost, st));
    MCX_CUDA(cudaStreamSynchronize(st));
    return MCX_OK;
}

MCX_API mcx_status mcx_graph_init_random(mcx_graph* g, uint64_t seed, uint32_t stream) {
    if (!g) return fail(MCX_ERR_INVALID_ARG, "graph is NULL");
    const int grid = (int)std::min<long long>((g->n + 255) / 256, (long long)g->ctx->num_sms * 8);
    k_graph_init_random<<<grid, 256, 0, g->ctx->stream>>>(g->d_perm, g->n, g->d_spins, (uint32_t)seed,
                                                          (uint32_t)(seed >> 32), stream, g->bc ? 1 : 0);
    count_launch(g->ctx);
    MCX_CUDA(cudaGetLastError());
    return graph_recompute(g);
}

MCX_API mcx_status mcx_graph_init_uniform(mcx_graph* g, int8_t value) {
    if (!g) return fail(MCX_ERR_INVALID_ARG, "graph is NULL");
    if (value != 1 && value != -1 && !(g->bc && value == 0))
        return fail(MCX_ERR_INVALID_ARG, "value %d is not a spin state of this model", (int)value);
    const int grid = (int)std::min<long long>((g->n + 255) / 256, (long long)g->ctx->num_sms * 8);
    k_graph_init_uniform<<<grid, 256, 0, g->ctx->stream>>>(g->d_perm, g->n, g->d_spins, value);
    count_launch(g->ctx);
    MCX_CUDA(cudaGetLastError());
    return graph_recompute(g);
}

MCX_API mcx_status mcx_graph_energy(mcx_graph* g, int full, double* energy, int64_t* magnetization) {
    if (!g) return fail(MCX_ERR_INVALID_ARG, "graph is NULL");
    if (full) MCX_CHECK(graph_recompute(g));
    double E = 0.0;
    long long M = 0;
    cudaStream_t st = g->ctx->stream;
    MCX_CUDA(cudaMemcpyAsync(&E, g->d_E, sizeof(E), cudaMemcpyDeviceToHost, st));
    MCX_CUDA(cudaMemcpyAsync(&M, g->d_M, sizeof(M), cudaMemcpyDeviceToHost, st));
    MCX_CUDA(cudaStreamSynchronize(st));
    if (energy) *energy = E;
    if (magnetization) *magnetization = M;
    return MCX_OK;
}

static mcx_status graph_site(mcx_graph* g, int64_t i, int target, int op, double* out) {
    if (!g) return fail(MCX_ERR_INVALID_ARG, "graph is NULL");
    if (i < 0 || i >= g->n) return fail(MCX_ERR_OUT_OF_RANGE, "site %lld outside 0..%lld", (long long)i,
                                        (long long)g->n - 1);
    int32_t p = 0;
    cudaStream_t st = g->ctx->stream;
    MCX_CUDA(cudaMemcpyAsync(&p, g->d_perm + i, sizeof(p), cudaMemcpyDeviceToHost, st));
    MCX_CUDA(cudaStreamSynchronize(st));
    const GraphDev d = g->dev(0.0);
    if (g->edgej) site_launch<true>(g->bc, g->field, st, d, p, target, op, g->d_site);
    else site_launch<false>(g->bc, g->field, st, d, p, target, op, g->d_site);
    count_launch(g->ctx);
    MCX_CUDA(cudaGetLastError());
    double v = 0.0;
    MCX_CUDA(cudaMemcpyAsync(&v, g->d_site, sizeof(v), cudaMemcpyDeviceToHost, st));
    MCX_CUDA(cudaStreamSynchronize(st));
    if (out) *out = v;
    return MCX_OK;
}

MCX_API mcx_status mcx_graph_delta_energy(mcx_graph* g, int64_t i, double* delta_energy) {
    if (g && g->bc) return fail(MCX_ERR_INVALID_ARG, "a Blume-Capel site needs the new state: mcx_graph_delta_energy_to");
    return graph_site(g, i, 2, 0, delta_energy);
}

MCX_API mcx_status mcx_graph_flip(mcx_graph* g, int64_t i) {
    if (g && g->bc) return fail(MCX_ERR_INVALID_ARG, "a Blume-Capel site needs the new state: mcx_graph_set_site");
    return graph_site(g, i, 2, 1, nullptr);
}

MCX_API mcx_status mcx_graph_delta_energy_to(mcx_graph* g, int64_t i, int8_t s_new, double* delta_energy) {
    if (!g) return fail(MCX_ERR_INVALID_ARG, "graph is NULL");
    if (s_new < -1 || s_new > 1 || (!g->bc && s_new == 0))
        return fail(MCX_ERR_INVALID_ARG, "%d is not a spin state of this model", (int)s_new);
    return graph_site(g, i, s_new, 0, delta_energy);
}

MCX_API mcx_status mcx_graph_set_site(mcx_graph* g, int64_t i, int8_t s_new) {
    if (!g) return fail(MCX_ERR_INVALID_ARG, "graph is NULL");
    if (s_new < -1 || s_new > 1 || (!g->bc && s_new == 0))
        return fail(MCX_ERR_INVALID_ARG, "%d is not a spin state of this model", (int)s_new);
    return graph_site(g, i, s_new, 1, nullptr);
}

MCX_API mcx_status mcx_graph_spin_flip(mcx_graph* g, mcx_algorithm alg, double beta, mcx_rng* rng, int64_t nattempts,
                                       mcx_counters* counters) {
    if (!g || !rng) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (alg < MCX_METROPOLIS || alg > MCX_HEATBATH) return fail(MCX_ERR_INVALID_ARG, "unknown algorithm %d", (int)alg);
    if (nattempts < 0) return fail(MCX_ERR_INVALID_ARG, "nattempts < 0");
    if (!std::isfinite(beta)) return fail(MCX_ERR_INVALID_ARG, "beta must be finite");
    if (nattempts == 0) return MCX_OK;
    mcx_ctx* ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    void* scratch = nullptr;  // (attempts, accepted) of this call
    MCX_CHECK(ctx_scratch(ctx, 2 * sizeof(unsigned long long), &scratch));
    GraphDev d = g->dev(beta);
    const int32_t* perm = g->d_perm;
    long long n = g->n, nat = nattempts;
    int ialg = (int)alg;
    uint32_t k0 = (uint32_t)rng->seed, k1 = (uint32_t)(rng->seed >> 32), sid = rng->stream;
    unsigned long long a0 = rng->counter;
    unsigned long long* counts = static_cast<unsigned long long*>(scratch);
    void* args[] = {&d, &perm, &n, &ialg, &k0, &k1, &sid, &a0, &nat, &counts};
    cudaError_t e;
    if (g->edgej) e = g->bc ? seq_launch<true, true>(g->field, st, args) : seq_launch<true, false>(g->field, st, args);
    else e = g->bc ? seq_launch<false, true>(g->field, st, args) : seq_launch<false, false>(g->field, st, args);
    count_launch(ctx);
    MCX_CUDA(e);
    rng->counter += (uint64_t)nattempts;
    if (counters) {
        unsigned long long h[2];
        MCX_CUDA(cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, st));
        MCX_CUDA(cudaStreamSynchronize(st));
        counters->attempts += h[0];
        counters->accepted += h[1];
    }
    return MCX_OK;
}

MCX_API mcx_status mcx_graph_sweep(mcx_graph* g, mcx_algorithm alg, double beta, mcx_rng* rng, int64_t nsweeps,
                                   double* E_series, int64_t* M_series, mcx_counters* counters) {
    if (!g || !rng) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (alg < MCX_METROPOLIS || alg > MCX_HEATBATH) return fail(MCX_ERR_INVALID_ARG, "unknown algorithm %d", (int)alg);
    if (nsweeps < 0) return fail(MCX_ERR_INVALID_ARG, "nsweeps < 0");
    if (!std::isfinite(beta)) return fail(MCX_ERR_INVALID_ARG, "beta must be finite");
    if (nsweeps == 0) return MCX_OK;
    mcx_ctx* ctx = g->ctx;
    cudaStream_t st = ctx->stream;
    const bool table = g->table_mode();
    if (table) MCX_CHECK(graph_table(g, alg, beta));
    // the series always stays on the device (autocorrelation times read it in place)
    if (nsweeps > g->ser_cap) {
        if (g->d_Eser) gfree(g, g->d_Eser);
        if (g->d_Mser) gfree(g, g->d_Mser);
        g->d_Eser = nullptr;
        g->d_Mser = nullptr;
        g->ser_cap = 0;
        MCX_CHECK(galloc(g, &g->d_Eser, (size_t)nsweeps));
        MCX_CHECK(galloc(g, &g->d_Mser, (size_t)nsweeps));
        g->ser_cap = nsweeps;
    }
    const SweepFns fns = g->bc ? bc_sweep_fns(alg, table, g->edgej, g->field) : sweep_fns(alg, table, g->edgej, g->field);
    MCX_CUDA(cudaMemsetAsync(g->d_acc, 0, sizeof(unsigned long long), st));
    const GraphDev d = g->dev(beta);
    const uint32_t k0 = (uint32_t)rng->seed, k1 = (uint32_t)(rng->seed >> 32);
    if (g->npad <= kSmallGraph) {
        fns.small<<<1, fns.small_threads, (size_t)g->npad, st>>>(d, g->d_classes, g->ncol, k0, k1, rng->stream,
                                                            rng->counter, nsweeps, g->d_Eser,
                                                            g->d_Mser, (int)g->npad);
        count_launch(ctx);
    } else {
        int bps = 0;
        MCX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fns.cls, kGraphBlock, 0));
        bps = std::max(1, std::min(bps, 8));
        MCX_CUDA(cudaMemsetAsync(g->d_part, 0, sizeof(double) * (size_t)g->nparts, st));
        // every launch after the first depends programmatically on the one before: the
        // kernels read nothing before pdl_wait, which waits for the previous grid (and so,
        // one grid at a time, for every earlier one)
        cudaLaunchAttribute pdl[1];
        pdl[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        pdl[0].val.programmaticStreamSerializationAllowed = 1;
        cudaLaunchConfig_t cfg = {};
        cfg.blockDim = dim3(kGraphBlock);
        cfg.stream = st;
        cfg.attrs = pdl;
        for (int64_t t = 0; t < nsweeps; ++t) {
            const unsigned long long sweep = rng->counter + (unsigned long long)t;
            for (size_t ci = 0; ci < g->classes.size(); ++ci) {
                const GClass& c = g->classes[ci];
                const int grid = (int)std::min<long long>((c.nslices + 2 * kSlicesPerBlock - 1) / (2 * kSlicesPerBlock),
                                                          (long long)ctx->num_sms * bps);
                cfg.gridDim = dim3((unsigned)std::max(grid, 1));
                cfg.numAttrs = (t == 0 && ci == 0) ? 0 : 1;
                MCX_CUDA(cudaLaunchKernelEx(&cfg, fns.cls, d, c, k0, k1, rng->stream, sweep));
            }
            cfg.gridDim = dim3(1);
            cfg.numAttrs = 1;
            MCX_CUDA(cudaLaunchKernelEx(&cfg, k_graph_finish, g->d_part, g->nparts, g->d_E, (const long long*)g->d_M,
                                        g->d_Eser, g->d_Mser, (long long)t));
            count_launch(ctx, (uint64_t)g->classes.size() + 1);
        }
    }
    MCX_CUDA(cudaGetLastError());
    rng->counter += (uint64_t)nsweeps;
    g->ser_len = nsweeps;
    if (counters || E_series || M_series) {
        unsigned long long acc1 = 0;
        MCX_CUDA(cudaMemcpyAsync(&acc1, g->d_acc, sizeof(acc1), cudaMemcpyDeviceToHost, st));
        if (E_series)
            MCX_CUDA(cudaMemcpyAsync(E_series, g->d_Eser, sizeof(double) * (size_t)nsweeps, cudaMemcpyDeviceToHost, st));
        if (M_series)
            MCX_CUDA(cudaMemcpyAsync(M_series, g->d_Mser, sizeof(long long) * (size_t)nsweeps, cudaMemcpyDeviceToHost,
                                     st));
        MCX_CUDA(cudaStreamSynchronize(st));
        if (counters) {
            counters->attempts += (uint64_t)g->n * (uint64_t)nsweeps;
            counters->accepted += acc1;
        }
    }
    return MCX_OK;
}

MCX_API mcx_status mcx_graph_tau_int(mcx_graph* g, int quantity, int64_t max_lag, double c, double* tau) {
    if (!g || !tau) return fail(MCX_ERR_INVALID_ARG, "NULL argument");
    if (quantity != 0 && quantity != 1) return fail(MCX_ERR_INVALID_ARG, "quantity must be 0 (energy) or 1 (magnetization)");
    if (!(c > 0)) return fail(MCX_ERR_INVALID_ARG, "c must be positive");
    const long long n = g->ser_len;
    if (n < 2) return fail(MCX_ERR_INVALID_ARG, "the last sweep call recorded %lld sweeps (at least 2 needed)", n);
    if (max_lag > n / 2) return fail(MCX_ERR_INVALID_ARG, "max_lag must satisfy 1 <= max_lag <= floor(n/2)");
    std::vector<TraceSrc> srcs(1);
    TraceSrc& s = srcs[0];
    s = TraceSrc{};
    s.stride = 1;
    if (quantity == 0) {
        s.base = g->d_Eser;
        s.type = TRACE_F64;
    } else {
        s.base = g->d_Mser;
        s.type = TRACE_I64;
        s.ncols = 1;
        s.coef[0] = 1.0;
    }
    tau_window(s, n, 2, max_lag);
    return launch_tau_int(g->ctx, srcs, nullptr, 0, c, tau);
}

}  // extern "C"

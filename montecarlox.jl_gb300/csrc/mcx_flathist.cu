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
// change is fixed in advance (its neighbours are all of the other colour): one warp
// of the walker's block produces proposals, energy changes and log-uniforms for
// batches of 32 sites while the other warp's lane 0 runs the short dependent scan
// over the previous batches in site order.  Throughput comes from many walkers (one
// block each), the pattern of the reference's parallel multicanonical walkers.
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

// Each walker is one block of two warps.  The producer warp computes, for batches of
// 32 consecutive sites of the current colour, the proposals, energy changes and
// single-precision brackets of log(U) into a ring of kFHSlots shared-memory slots;
// the consumer warp's lane 0 runs the dependent scan over each batch in site order,
// then its 32 lanes write the accepted spins.  Within one colour every energy change
// is fixed in advance (all neighbours are of the other colour), so the producer runs
// ahead of the scan; at a colour boundary it waits until the consumer has written the
// last batch.  Hand-offs use named barriers (FULL / EMPTY per slot, COL per colour)
// that both warps pass in the same sequence whatever happens, so none can wait forever.
constexpr int kFHSlots = 4;
constexpr int kFHBarFull = 1, kFHBarEmpty = 5, kFHBarCol = 9;

// Each walker keeps a window of kFHWin log-weights around its current bin in shared
// memory (FP64 and a single-precision copy relative to a centre value), so the scan
// never waits on a global load; the window moves when a proposed bin falls outside
// it (Wang-Landau writes the window back first).  Histogram counts of the window
// accumulate in shared memory and go to global memory when the window moves.
constexpr int kFHWin = 512;
// Guard entries on both sides of the single-precision window: one move changes the bin
// by less than kFHWin / 2 (fh_window_ok), so a proposal from a bin inside the window
// indexes fwin(sh) within [-kFHGuard, kFHWin + kFHGuard) without a bounds select.
constexpr int kFHGuard = kFHWin / 2;
// Bound on |logf(float(U)) - 53 ln 2 (in float) - log(U)|: float(k) is within 2^-24
// relative of k, logf within 1 ulp (<= 2^-18 for results below 64 in magnitude), the
// float constant and subtraction within 2^-18 each: far below 2^-14.
constexpr double kLogMargin = 6.103515625e-05;  // 2^-14

struct FHSlot {
    // producer -> consumer
    int4 cand[32];                // dE, lo, hacc (float bits), packed (sn, ds, dq, dp)
    unsigned long long k53[32];   // U = k * 2^-53
    long long j0;                 // first site of the batch in its colour
    int colour;
    // consumer -> producer (applied when the slot is next reused or at a colour end)
    int bin[32];                  // bin after each attempt, relative to base
    long long base;
    unsigned int accmask;         // accepted attempts
    int nproc;                    // attempts made (fewer than the batch after a range stop)
    int pending;                  // results not applied yet
};

struct FHShared {
    FHSlot slot[kFHSlots];
    double win[kFHWin];
    float fwin_g[kFHGuard + kFHWin + kFHGuard];  // fwin(sh)[-kFHGuard, kFHWin + kFHGuard)
    uint32_t rnd[3][8][4];  // producer: Philox blocks of one batch by purpose
    uint8_t accf[32];       // consumer: 1 where the batch's attempt was accepted
    float2 thr2[32];        // consumer: (hacc + ew, lo - ew) of the batch's sites
    int stop;
};

__device__ __forceinline__ float* fwin(FHShared& sh) { return sh.fwin_g + kFHGuard; }

__device__ __forceinline__ void fh_bar_sync(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }
__device__ __forceinline__ void fh_bar_arrive(int id) { asm volatile("bar.arrive %0, 64;" ::"r"(id) : "memory"); }

__device__ __forceinline__ long long fh_window_base(long long b, long long nbins) {
    long long wb = b - kFHWin / 2;
    if (wb > nbins - kFHWin) wb = nbins - kFHWin;
    return wb < 0 ? 0 : wb;
}

// Absolute margin for the single-precision decision: with B >= |fwin[i]| over the
// window, d = fl(fa - fb) is within 2^-22 * B of the FP64 difference lr (two rounded
// conversions and one rounded subtraction), and forming the thresholds fl(h +- ew)
// rounds by at most 2^-24 (|h| + ew) with |h| < 40.  So d > fl(hacc + ew) proves
// lr > hacc and d <= fl(lo - ew) proves lr < lo whenever ew >= 2^-21 (B + 40);
// (B + 64) 2^-20 is used.  A window holding a value that is not finite in single
// precision gets NaN, which sends every decision to FP64.
__device__ __forceinline__ float fh_margin(float B) {
    return B <= 3.0e38f ? (B + 64.0f) * 9.5367431640625e-07f : __int_as_float(0x7FC00000);
}

// x * 2^e as an integer when that is exact and below 2^52 in magnitude (the range in which
// FP64 sums of such values are exact), else false.
__device__ __forceinline__ bool fh_units(double x, int e, long long& n) {
    const double y = ldexp(x, e);
    if (!(fabs(y) < 4503599627370496.0)) return false;  // 2^52; false for NaN
    n = (long long)y;
    return (double)n == y;
}

// Loads the window at wb (all lanes of the consumer); returns the margin.  With g.wl_exact
// and every value (and the centre) a multiple of logf = 2^-wl_exp in range, the window is
// held as integers in units of logf (`exact`, icw = the centre in those units); the single-
// precision copy is the same either way.
__device__ __forceinline__ float fh_window_load(FHShared& sh, const FHGeom& g, const double* lnw, long long wb,
                                                long long centre, int lane, double& c, int& exact, long long& icw) {
    const long long nbins = g.nbins;
    const double v = lnw[centre];
    c = (v - v == 0.0) ? v : 0.0;  // v finite ? v : 0
    unsigned int m = 0;
    for (int i = lane; i < kFHWin; i += 32) {
        const double x = wb + i < nbins ? lnw[wb + i] : 0.0;
        const float f = (float)(x - c);
        sh.win[i] = x;
        fwin(sh)[i] = f;
        const unsigned int a = __float_as_uint(f) & 0x7FFFFFFFu;  // |f|; NaN / inf above every finite
        m = a > m ? a : m;
    }
    exact = 0;
    if (g.wl_exact) {  // Wang-Landau: the integer form when every value allows it
        bool ok = fh_units(c, g.wl_exp, icw);
        long long n = 0;
        for (int i = lane; i < kFHWin; i += 32) ok = ok && fh_units(sh.win[i], g.wl_exp, n);
        exact = __all_sync(0xFFFFFFFFu, ok) ? 1 : 0;
        if (exact) {
            long long* iw = reinterpret_cast<long long*>(sh.win);
            for (int i = lane; i < kFHWin; i += 32) iw[i] = (long long)ldexp(sh.win[i], g.wl_exp);
        }
    }
    m = __reduce_max_sync(0xFFFFFFFFu, m);
    __syncwarp();
    return fh_margin(__uint_as_float(m));
}


__device__ __forceinline__ void fh_window_store(const FHShared& sh, const FHGeom& g, double* lnw, long long wb,
                                                int lane, int exact) {
    __syncwarp();
    const long long* iw = reinterpret_cast<const long long*>(sh.win);
    for (int i = lane; i < kFHWin; i += 32)
        if (wb + i < g.nbins) lnw[wb + i] = exact ? ldexp((double)iw[i], -g.wl_exp) : sh.win[i];
    __syncwarp();
}

// Producer, stage 1: the raw spins one lane needs for site j0 + lane of colour c (own
// spin and 2*dim neighbours), loaded one batch ahead so that their latency overlaps the
// previous batch's arithmetic and the wait for a free slot.
struct FHLoad {
    int so;
    int nb[6];
};

__device__ __forceinline__ FHLoad fh_load(const FHGeom& g, const int8_t* cur, const int8_t* oth, int c, long long j0,
                                          int r0, int q0, long long ncol, int lane) {
    FHLoad L;
    L.so = 0;
#pragma unroll
    for (int d = 0; d < 6; ++d) L.nb[d] = 0;
    const long long j = j0 + lane;
    if (j < ncol) {
        int q = q0 + lane, r = r0;
        while (q >= g.W) {
            q -= g.W;
            ++r;
        }
        int y = r, z = 0;
        if (g.dim == 3) {
            z = r / g.Ly;
            y = r - z * g.Ly;
        }
        const RowInfo ri = row_info_yz(y, z, g.Ly, g.Lz, c, g.dim);
        const int qs = ri.p == 0 ? (q == 0 ? g.W - 1 : q - 1) : (q == g.W - 1 ? 0 : q + 1);
        L.so = cur[j];
        L.nb[0] = oth[j];
        L.nb[1] = oth[(long long)r * g.W + qs];
        L.nb[2] = oth[ri.ryp * g.W + q];
        L.nb[3] = oth[ri.rym * g.W + q];
        if (g.dim == 3) {
            L.nb[4] = oth[ri.rzp * g.W + q];
            L.nb[5] = oth[ri.rzm * g.W + q];
        }
    }
    return L;
}

// Producer, stage 2: candidates of one batch (32 sites of colour c from site j0).
__device__ __forceinline__ void fh_produce(FHShared& sh, FHSlot& sl, const FHGeom& g, const FHLoad& L, int c,
                                           unsigned long long t, long long j0, long long ncol, uint32_t k0,
                                           uint32_t k1, uint32_t stream, int lane) {
    // one Philox block per lane: purpose lane / 8 (accept, low word, proposal), group lane % 8
    {
        const int pur = lane >> 3, grp = lane & 7;
        if (pur < 2 + g.model) {
            const uint32_t p = pur == 0 ? P_ACCEPT : (pur == 1 ? P_LOW : P_PROPOSE);
            const uint4 v = philox10(make_uint4((uint32_t)((j0 >> 2) + grp), (uint32_t)t, ctr_word2(t, c, p), stream),
                                     k0, k1);
            sh.rnd[pur][grp][0] = v.x;
            sh.rnd[pur][grp][1] = v.y;
            sh.rnd[pur][grp][2] = v.z;
            sh.rnd[pur][grp][3] = v.w;
        }
    }
    __syncwarp();
    int4 cd = make_int4(0, 0, 0, 0);
    unsigned long long k53 = 0;
    if (j0 + lane < ncol) {
        const int so = L.so;
        const int S = L.nb[0] + L.nb[1] + L.nb[2] + L.nb[3] + L.nb[4] + L.nb[5];
        const int grp = lane >> 2, wd = lane & 3;
        const int sn = g.model == 0 ? -so : bc_propose(so, (int)(sh.rnd[2][grp][wd] >> 31));
        const int ds = sn - so, dq = sn * sn - so * so, dp = ds * S;
        const long long dE = -g.J * dp + g.D * dq - g.h * ds;
        k53 = ((unsigned long long)sh.rnd[0][grp][wd] << 21) | (unsigned long long)(sh.rnd[1][grp][wd] >> 11);
        // single-precision log(U) and a margin that bounds its distance to the FP64
        // log of the decision rule (logf: <= 1 ulp, |log U| < 37.5)
        const float l32 = logf(__ull2float_rn(k53)) - 36.7368005696771f;  // 53 ln 2
        const float lo = l32 - (float)kLogMargin;
        const float hacc = fminf(l32 + (float)kLogMargin, 0.0f);  // accept when lr > min(0, log U)
        cd = make_int4((int)dE, __float_as_int(lo), __float_as_int(hacc),
                       (int)((uint32_t)(uint8_t)sn | ((uint32_t)(uint8_t)ds << 8) | ((uint32_t)(uint8_t)dq << 16) |
                             ((uint32_t)(uint8_t)dp << 24)));
    }
    sl.cand[lane] = cd;
    sl.k53[lane] = k53;
    __syncwarp();
}

// Consumer lane-0 state of one walker.
struct FHScan {
    long long E;   // energy (tracked when !FAST)
    long long Ewb; // start + wb * step
    int er;        // E - Ewb (tracked when FAST)
    int bi;        // current bin, relative to wb
    float flwo;    // fwin[bi]
    float ew;      // decision margin of the window
    double cw;     // centre of the single-precision window copy
    int exact;     // the window holds ln g in integer units of logf (Wang-Landau)
    long long icw; // cw in those units
    unsigned long long steps;
};

// Scans sites i..n-1 of one batch (consumer lane 0).  Stops early with `need` set to
// the bin that must come into the window, or with status 2 (energy out of range).
template <bool FAST>
__device__ __forceinline__ void fh_scan(FHShared& sh, FHSlot& sl, const FHGeom& g, long long wb, int lim,
                                        FHScan& st, int& i, int n, long long& need, int& status) {
    const bool wl = g.mode == 1;
    int4 nx = sl.cand[i < n ? i : 0];
    for (; i < n; ++i) {
        const int4 cd = nx;
        if (i + 1 < n) nx = sl.cand[i + 1];  // prefetch: keeps the load off the dependent chain
        int bn;
        long long En = 0;
        int en = 0;
        if (FAST) {
            en = st.er + cd.x;
            if ((unsigned)en < (unsigned)lim) {
                bn = en >> g.shift;
            } else {
                long long b;
                if (!fh_bin(st.Ewb + en, g, b)) {
                    status = 2;
                    break;
                }
                if (b < wb || b >= wb + kFHWin) {
                    need = b;
                    break;
                }
                bn = (int)(b - wb);
            }
        } else {
            En = st.E + cd.x;
            long long b;
            if (!fh_bin(En, g, b)) {
                status = 2;
                break;
            }
            if (b < wb || b >= wb + kFHWin) {
                need = b;
                break;
            }
            bn = (int)(b - wb);
        }
        // lr = lnw[bn] - lnw[bo] against log(U), decided in single precision when the
        // margins allow, else in FP64 with the project's log
        const float fa = fwin(sh)[bn];
        const float d = fa - st.flwo;
        bool acc;
        if (d > __int_as_float(cd.z) + st.ew) acc = true;
        else if (d <= __int_as_float(cd.y) - st.ew) acc = false;
        else {
            const long long* iw = reinterpret_cast<const long long*>(sh.win);
            const double lr = st.exact ? ldexp((double)(iw[bn] - iw[st.bi]), -g.wl_exp) : sh.win[bn] - sh.win[st.bi];
            acc = (lr > 0.0) || (mcx_log((double)sl.k53[i] * 1.1102230246251565404236316680908203125e-16) < lr);
        }
        if (acc) {
            sh.accf[i] = 1;
            st.bi = bn;
            if (FAST) st.er = en;
            else st.E = En;
            st.flwo = fa;
        }
        if (wl) {
            float f;
            if (st.exact) {  // ln g -= logf is a decrement in units of logf, exact like the FP64 one
                long long* iw = reinterpret_cast<long long*>(sh.win);
                const long long n = iw[st.bi] - 1;
                iw[st.bi] = n;
                // = (float)(v - cw): rounding n - icw, then scaling by 2^-wl_exp, which is exact
                f = __ll2float_rn(n - st.icw) * __int_as_float((127 - g.wl_exp) << 23);
            } else {
                const double v = sh.win[st.bi] - g.logf;
                sh.win[st.bi] = v;
                f = (float)(v - st.cw);
            }
            fwin(sh)[st.bi] = f;
            st.flwo = f;
            // keep the margin valid for the changed value (NaN stays NaN)
            const float m = fh_margin(fabsf(f));
            if (st.ew == st.ew && !(m <= st.ew)) st.ew = m;
        }
        sl.bin[i] = st.bi;
    }
}

// Multicanonical scan with power-of-two bins (consumer lane 0): straight-line code while
// every proposed bin is inside the window and the single-precision decision is clear
// (thresholds precomputed in thr2); the next site's energy change and thresholds are
// loaded one site ahead, so the dependent chain per site is one shared-memory load of
// the weight plus a handful of integer and float operations.  Returns at the first
// site that needs fh_scan (window miss, range end, FP64 decision) or at the end of the
// batch.
__device__ __forceinline__ void fh_scan_fast(FHShared& sh, FHSlot& sl, int shift, int lim, FHScan& st, int& i,
                                             int n) {
    if (i >= n) return;
    int er = st.er, bi = st.bi;
    float flwo = st.flwo;
    int k = i;
    int dn = sl.cand[k].x;
    float2 t = sh.thr2[k];
    bool go = true;
    while (go) {
        const int en = er + dn;
        const bool ok = (unsigned)en < (unsigned)lim;
        const int b = ok ? (en >> shift) : bi;
        const float fa = fwin(sh)[b];
        const int kn = k + 1 < 32 ? k + 1 : 31;
        const int dn2 = sl.cand[kn].x;
        const float2 t2 = sh.thr2[kn];
        const float d = fa - flwo;
        const bool acc = d > t.x;
        const bool clear = ok && (acc || d <= t.y);
        if (clear) {
            if (acc) {
                er = en;
                bi = b;
                flwo = fa;
            }
            sh.accf[k] = (uint8_t)acc;
            sl.bin[k] = bi;
            ++k;
            dn = dn2;
            t = t2;
        }
        go = clear && k < n;
    }
    i = k;
    st.er = er;
    st.bi = bi;
    st.flwo = flwo;
}

// Branch-free Multicanonical pass over a full batch of 32 sites (consumer lane 0), used while the
// current bin is inside the window: every site is decided in single precision with
// fa > fl(flwo + hacc + ew) (accept) or fa <= fl(flwo + lo - ew) (reject), which the same
// margin proves equal to the FP64 rule.  No site depends on a branch, so the dependent
// chain per site is an add, the window load, a compare and a select.  A site that falls
// outside the window or is not clear in single precision makes the pass report false;
// the caller then redoes the batch with fh_scan_fast / fh_scan, which overwrite
// everything this pass wrote.  Moves are taken only inside the window, so every load
// stays within the guard entries.
__device__ __forceinline__ bool fh_batch_fast(FHShared& sh, FHSlot& sl, int shift, int lim, FHScan& st,
                                              unsigned int& mask_out) {
    const float* fw = fwin(sh);
    int er = st.er, bi = st.bi;
    float flwo = st.flwo;
    unsigned int mask = 0;
    bool clear = true;
#pragma unroll
    for (int q = 0; q < 32; ++q) {
        {
            const int en = er + sl.cand[q].x;
            const int b = en >> shift;
            const float fa = fw[b];
            const float2 t = sh.thr2[q];
            const float ta = flwo + t.x, tr = flwo + t.y;
            const bool ok = (unsigned)en < (unsigned)lim;
            const bool up = fa > ta;
            const bool acc = up & ok;
            clear = clear & ok & (up | (fa <= tr));
            er = acc ? en : er;
            bi = acc ? b : bi;
            flwo = acc ? fa : flwo;
            mask |= acc ? (1u << q) : 0u;
            sl.bin[q] = bi;
        }
    }
    if (!clear) return false;
    st.er = er;
    st.bi = bi;
    st.flwo = flwo;
    mask_out = mask;
    return true;
}

// Decision thresholds of the batch for the current window margin (all lanes).
__device__ __forceinline__ void fh_thresholds(FHShared& sh, const FHSlot& sl, float ew, int lane) {
    const int4 c = sl.cand[lane];
    sh.thr2[lane] = make_float2(__int_as_float(c.z) + ew, __int_as_float(c.y) - ew);
    __syncwarp();
}

// Producer: applies the consumer's results of one batch (all lanes): histogram counts
// of the bins after each attempt (lanes holding the same bin add once, as a group), the
// accepted spins and the observable deltas.
__device__ __forceinline__ void fh_apply(FHSlot& sl, int8_t* col0, int8_t* col1, unsigned long long* H, long long& dP,
                                         long long& dM, long long& dQ, int lane) {
    const bool act = lane < sl.nproc;
    const unsigned int am = __ballot_sync(0xFFFFFFFFu, act);
    if (act) {
        const long long bin = sl.base + sl.bin[lane];
        const unsigned int grp = __match_any_sync(am, bin);
        if (lane == __ffs(grp) - 1) atomicAdd(&H[bin], (unsigned long long)__popc(grp));
        if ((sl.accmask >> lane) & 1u) {
            const uint32_t pk = (uint32_t)sl.cand[lane].w;
            (sl.colour ? col1 : col0)[sl.j0 + lane] = (int8_t)(pk & 0xFFu);
            dP += (int8_t)(pk >> 24);
            dM += (int8_t)((pk >> 8) & 0xFFu);
            dQ += (int8_t)((pk >> 16) & 0xFFu);
        }
    }
    __syncwarp();
    if (lane == 0) sl.pending = 0;
    __syncwarp();
}

__global__ void __launch_bounds__(64, 1) k_flathist(const FHArgs a) {
    __shared__ FHShared sh;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wid = blockIdx.x;
    if (wid >= a.nwalkers) return;  // whole block
    FHWalker& w = a.walkers[wid];
    const FHGeom g = w.g;
    int8_t* const col0 = w.col[0];
    int8_t* const col1 = w.col[1];
    const long long ncol = (long long)g.W * g.Ly * g.Lz;
    const long long nb = (ncol + 31) / 32;                // batches per colour
    const long long total = g.nsweeps * 2 * nb;          // batches of the launch
    const unsigned long long sweep0 = w.sweep0;
    if (warp == 0 && lane == 0) sh.stop = 0;
    if (threadIdx.x < kFHSlots) sh.slot[threadIdx.x].pending = 0;
    for (int i = threadIdx.x; i < kFHGuard + kFHWin + kFHGuard; i += 64) sh.fwin_g[i] = 0.0f;
    __syncthreads();

    if (warp == 0) {
        // ------------------------------------------------------------ producer --
        // Prepares batches, and applies the consumer's results of a batch when its slot
        // is reused or at the end of a colour: histogram counts, accepted spins and the
        // running (pair, spin, spin2) sums with the per-sweep series.
        const uint32_t k0 = w.k0, k1 = w.k1, stream = w.stream;
        unsigned long long* const H = w.H;
        long long* const series = w.series;
        long long P = w.P, M = w.M, Q = w.Q;
        if (w.state) {
            P = w.state[0];
            M = w.state[1];
            Q = w.state[2];
        }
        long long dP = 0, dM = 0, dQ = 0;
        bool stopped = false;
        // every slot with results not applied yet (the consumer has finished the colour)
        auto apply_all = [&]() {
            for (int k = 0; k < kFHSlots; ++k)
                if (sh.slot[k].pending) fh_apply(sh.slot[k], col0, col1, H, dP, dM, dQ, lane);
        };
        // fold the sweep's deltas; the series records sweeps that ran to the end
        auto end_sweep = [&](long long s) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                dP += __shfl_down_sync(0xFFFFFFFFu, dP, o);
                dM += __shfl_down_sync(0xFFFFFFFFu, dM, o);
                dQ += __shfl_down_sync(0xFFFFFFFFu, dQ, o);
            }
            dP = __shfl_sync(0xFFFFFFFFu, dP, 0);
            dM = __shfl_sync(0xFFFFFFFFu, dM, 0);
            dQ = __shfl_sync(0xFFFFFFFFu, dQ, 0);
            P += dP;
            M += dM;
            Q += dQ;
            dP = dM = dQ = 0;
            stopped = stopped || *(volatile int*)&sh.stop;
            if (lane == 0 && !stopped && series) {
                series[3 * s] = P;
                series[3 * s + 1] = M;
                series[3 * s + 2] = Q;
            }
        };
        long long qb = 0;
        for (long long s = 0; s < g.nsweeps; ++s) {
            const unsigned long long t = sweep0 + (unsigned long long)s;
            for (int c = 0; c < 2; ++c) {
                if (s > 0 || c > 0) {
                    fh_bar_sync(kFHBarCol);
                    apply_all();
                    if (c == 0) end_sweep(s - 1);
                }
                const int8_t* cur = c ? col1 : col0;
                const int8_t* oth = c ? col0 : col1;
                // spins of batches b and b + 1 are in registers or in flight; the loads of
                // batch b + 2 are issued after batch b is handed over, so the fence before
                // the hand-over never waits on them (sites the consumer has not reached)
                int r2 = 0, q2 = 0;  // row and column of the first site of the batch loaded next
                auto advance = [&]() {
                    q2 += 32;
                    while (q2 >= g.W) {
                        q2 -= g.W;
                        ++r2;
                    }
                };
                FHLoad ld0 = fh_load(g, cur, oth, c, 0, r2, q2, ncol, lane);
                advance();
                FHLoad ld1 = fh_load(g, cur, oth, c, 32, r2, q2, ncol, lane);
                advance();
                for (long long b = 0; b < nb; ++b, ++qb) {
                    const int sl = (int)(qb % kFHSlots);
                    if (qb >= kFHSlots) {
                        fh_bar_sync(kFHBarEmpty + sl);
                        if (sh.slot[sl].pending) fh_apply(sh.slot[sl], col0, col1, H, dP, dM, dQ, lane);
                    }
                    if (!*(volatile int*)&sh.stop)
                        fh_produce(sh, sh.slot[sl], g, ld0, c, t, b * 32, ncol, k0, k1, stream, lane);
                    if (lane == 0) {
                        sh.slot[sl].j0 = b * 32;
                        sh.slot[sl].colour = c;
                    }
                    __threadfence_block();
                    fh_bar_arrive(kFHBarFull + sl);
                    ld0 = ld1;
                    ld1 = fh_load(g, cur, oth, c, (b + 2) * 32, r2, q2, ncol, lane);
                    advance();
                }
            }
        }
        if (g.nsweeps > 0) {
            fh_bar_sync(kFHBarCol);  // the consumer has finished the last colour
            apply_all();
            end_sweep(g.nsweeps - 1);
        }
        if (lane == 0) {
            // a stopped sweep still folds the accepted moves made before the stop
            w.P = P;
            w.M = M;
            w.Q = Q;
            if (w.state) {
                w.state[0] = P;
                w.state[1] = M;
                w.state[2] = Q;
            }
        }
        return;
    }

    // ---------------------------------------------------------------- consumer --
    double* const lnw = w.lnw;
    int status = 0;
    FHScan st;
    {
        long long P = w.P, M = w.M, Q = w.Q;
        if (w.state) {
            P = w.state[0];
            M = w.state[1];
            Q = w.state[2];
        }
        st.E = -g.J * P + g.D * Q - g.h * M;
    }
    long long bo = 0;
    if (!fh_bin(st.E, g, bo)) status = 2;
    const bool fast = g.shift >= 0 && g.shift <= 20;
    long long wb = fh_window_base(status ? 0 : bo, g.nbins);
    int exact = 0;  // the window's integer form (all lanes)
    st.ew = fh_window_load(sh, g, lnw, wb, status ? 0 : bo, lane, st.cw, exact, st.icw);
    st.exact = exact;
    st.Ewb = g.start + wb * g.step;
    st.er = (int)(st.E - st.Ewb);
    st.bi = status ? 0 : (int)(bo - wb);
    st.flwo = fwin(sh)[st.bi];
    st.steps = 0;
    const bool muca_fast = fast && g.mode == 0;
    if (status && lane == 0) sh.stop = 1;
    unsigned long long accepted = 0;
    long long qb = 0;
    for (long long s = 0; s < g.nsweeps; ++s) {
        for (int c = 0; c < 2; ++c) {
            for (long long b = 0; b < nb; ++b, ++qb) {
                const int slot = (int)(qb % kFHSlots);
                fh_bar_sync(kFHBarFull + slot);
                FHSlot& sl = sh.slot[slot];
                int i = 0;
                unsigned int accmask = 0;
                if (status == 0) {
                    const int n = (int)((ncol - b * 32) < 32 ? (ncol - b * 32) : 32);
                    unsigned int fastmask = 0;  // acceptances of a successful fh_batch_fast (lane 0)
                    sh.accf[lane] = 0;
                    if (muca_fast) fh_thresholds(sh, sl, __shfl_sync(0xFFFFFFFFu, st.ew, 0), lane);
                    __syncwarp();
                    for (;;) {
                        long long need = -1;
                        if (lane == 0) {
                            const long long vis = wb + kFHWin < g.nbins ? kFHWin : g.nbins - wb;
                            const int lim = (int)(vis << (fast ? g.shift : 0));
                            const int i0 = i;
                            if (muca_fast && i == 0 && n == 32 && (unsigned)st.er < (unsigned)lim &&
                                fh_batch_fast(sh, sl, g.shift, lim, st, fastmask)) {
                                i = n;
                            } else if (muca_fast) {
                                for (;;) {
                                    fh_scan_fast(sh, sl, g.shift, lim, st, i, n);
                                    if (i >= n) break;
                                    fh_scan<true>(sh, sl, g, wb, lim, st, i, i + 1, need, status);
                                    if (need >= 0 || status) break;
                                }
                            } else if (fast) {
                                fh_scan<true>(sh, sl, g, wb, lim, st, i, n, need, status);
                            } else {
                                fh_scan<false>(sh, sl, g, wb, lim, st, i, n, need, status);
                            }
                            st.steps += (unsigned long long)(i - i0);
                        }
                        need = __shfl_sync(0xFFFFFFFFu, need, 0);
                        i = __shfl_sync(0xFFFFFFFFu, i, 0);
                        if (need < 0) break;
                        // move the window around the proposed bin (the current bin stays
                        // inside: one move changes the bin by far less than half the window);
                        // the bins recorded so far in this batch are rebased on the new window
                        if (g.mode == 1) fh_window_store(sh, g, lnw, wb, lane, exact);
                        const long long bo_all = __shfl_sync(0xFFFFFFFFu, wb + st.bi, 0);
                        const long long wb_new = fh_window_base(need, g.nbins);
                        __syncwarp();
                        if (lane < i) sl.bin[lane] += (int)(wb - wb_new);
                        __syncwarp();
                        long long icw = 0;
                        const float ew = fh_window_load(sh, g, lnw, wb_new, need, lane, st.cw, exact, icw);
                        if (lane == 0) {
                            st.ew = ew;
                            st.exact = exact;
                            st.icw = icw;
                            st.er += (int)((wb - wb_new) * g.step);  // FAST only (wb moves < 2^11 bins)
                            st.Ewb = g.start + wb_new * g.step;
                            st.bi = (int)(bo_all - wb_new);
                            st.flwo = fwin(sh)[st.bi];
                        }
                        wb = wb_new;
                        if (muca_fast) fh_thresholds(sh, sl, ew, lane);
                    }
                    __syncwarp();
                    accmask = __ballot_sync(0xFFFFFFFFu, sh.accf[lane] != 0) | __shfl_sync(0xFFFFFFFFu, fastmask, 0);
                    status = __shfl_sync(0xFFFFFFFFu, status, 0);
                }
                if (lane == 0) {
                    accepted += __popc(accmask);
                    if (status) sh.stop = 1;
                    sl.accmask = accmask;
                    sl.nproc = i;
                    sl.base = wb;
                    sl.pending = 1;
                }
                __syncwarp();
                __threadfence_block();
                if (qb + kFHSlots < total) fh_bar_arrive(kFHBarEmpty + slot);
            }
            fh_bar_arrive(kFHBarCol);
        }
    }
    if (g.mode == 1) fh_window_store(sh, g, lnw, wb, lane, exact);
    if (lane == 0) {
        w.steps = st.steps;
        w.accepted = accepted;
        w.status = status;
    }
}

// lnw[b] -= log(H[b]) for H[b] > 0 (src/ensembles/multicanonical.jl:32-43)
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

mcx_status launch_flathist_on(mcx_ctx* ctx, cudaStream_t stream, FHWalker* d_walkers, int nwalkers) {
    FHArgs a;
    a.walkers = d_walkers;
    a.nwalkers = nwalkers;
    k_flathist<<<nwalkers, 64, 0, stream>>>(a);
    count_launch(ctx);
    MCX_CUDA(cudaGetLastError());
    return MCX_OK;
}

mcx_status launch_flathist(mcx_ctx* ctx, FHWalker* d_walkers, int nwalkers) {
    return launch_flathist_on(ctx, ctx->stream, d_walkers, nwalkers);
}

bool fh_window_ok(int dim, long long J, long long D, long long h, long long step) {
    const long long z = 2 * dim;
    const long long maxde = 2 * (J < 0 ? -J : J) * z + 2 * (h < 0 ? -h : h) + (D < 0 ? -D : D);
    return maxde < (1ll << 30) && maxde / step + 2 < kFHWin / 2;
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
    for (int i = 0; i < nwalkers; ++i) {
        FHWalker& w = hw[i];
        std::memset(&w, 0, sizeof(w));
        w.col[0] = lats[i]->d_col[0];
        w.col[1] = lats[i]->d_col[1];
        const mcx_flathist* f = fhs[nfh == 1 ? 0 : i];
        w.lnw = f->d_lnw;
        w.H = f->d_H;
        w.series = (long long*)lats[i]->d_series;
        w.state = (long long*)lats[i]->d_state;  // the kernel reads and updates (P, M, Q) in place
        w.sweep0 = rngs[i].counter;
        w.k0 = (uint32_t)rngs[i].seed;
        w.k1 = (uint32_t)(rngs[i].seed >> 32);
        w.stream = rngs[i].stream;
    }
    void* dw = nullptr;
    MCX_CHECK(ctx_scratch(ctx, hw.size() * sizeof(FHWalker), &dw));
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
    {
        int ex = 0;
        const double mant = std::frexp(logf, &ex);  // logf = mant * 2^ex
        if (g.mode == 1 && mant == 0.5 && 1 - ex >= 0 && 1 - ex <= 40) {
            g.wl_exact = 1;
            g.wl_exp = 1 - ex;  // logf = 2^-wl_exp
        }
    }
    g.nsweeps = nsweeps;
    for (auto& w : hw) w.g = g;
    cudaError_t e = cudaMemcpyAsync(dw, hw.data(), hw.size() * sizeof(FHWalker), cudaMemcpyHostToDevice, ctx->stream);
    FHArgs a;
    a.walkers = (FHWalker*)dw;
    a.nwalkers = nwalkers;
    if (e == cudaSuccess) {
        k_flathist<<<nwalkers, 64, 0, ctx->stream>>>(a);
        count_launch(ctx);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hw.data(), dw, hw.size() * sizeof(FHWalker), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "flat-histogram sweep");
    bool range = false;
    for (int i = 0; i < nwalkers; ++i) {
        const FHWalker& w = hw[i];
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

/*
 * mcx_oracle.c -- CPU oracle for the spin-flip hot path (TEST INFRASTRUCTURE ONLY).
 *
 * Restates, in plain C, the MonteCarloX.jl / SpinSystems algorithms that the CUDA
 * library accelerates.  Used only as the checker by the tests, smoke() and the
 * CPU-baseline leg of bench.py.  Compile with -ffp-contract=off: every FP64
 * decision must be evaluated with exactly the operations written here.
 *
 * Reference citations are paths inside the MonteCarloX.jl repository.
 */
#include "mcx_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* Philox purposes (counter word 2, bits 24..31) */
enum { P_ACCEPT = 0, P_PROPOSE = 1, P_LOW = 2, P_INIT = 3, P_EXCHANGE = 4, P_SEQ = 5, P_SEQ2 = 6,
       P_PLANES = 9, P_TAIL = 10 };

/* ---------------------------------------------------------------------------
 * Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2, 3",
 * SC'11): 10 rounds of two 32x32->64 multiplies with a Weyl key schedule.
 * ------------------------------------------------------------------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* The checkerboard stream: key = seed, counter = (site>>3, sweep lo, sweep hi16 |
 * colour<<16 | purpose<<24, stream); the site takes word (site>>1)&3.  Eight
 * consecutive linear sites hold four sites of each colour, so one call feeds four
 * same-colour sites. */
uint32_t orc_site_word(uint64_t seed, uint32_t stream, uint64_t sweep, int colour,
                       int purpose, uint64_t site) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {(uint32_t)(site >> 3), (uint32_t)sweep,
                       ((uint32_t)(sweep >> 32) & 0xFFFFu) | ((uint32_t)colour << 16) |
                           ((uint32_t)purpose << 24),
                       stream};
    uint32_t out[4];
    orc_philox4x32_10(ctr, key, out);
    return out[(site >> 1) & 3];
}

/* The Philox block of the checkerboard stream at counter word 0 = x. */
static void orc_cb_block(uint64_t seed, uint32_t stream, uint64_t sweep, int colour, int purpose, uint32_t x,
                         uint32_t out[4]) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t ctr[4] = {x, (uint32_t)sweep,
                       ((uint32_t)(sweep >> 32) & 0xFFFFu) | ((uint32_t)colour << 16) | ((uint32_t)purpose << 24),
                       stream};
    orc_philox4x32_10(ctr, key, out);
}

/* The bit-plane uniform (the library's MCX_UNIFORMS_PLANES form) of the site with index e
 * among the sites of its colour (e = linear index >> 1; Lx a multiple of 128, so every
 * 64 consecutive e share one row): bits 31..24 are bit e & 63 of planes 0..7, where
 * plane 2j is words 0 | 1 << 32 and plane 2j+1 words 2 | 3 << 32 of the block at counter
 * (e >> 6) * 16 + j, purpose P_PLANES; bits 23..0 are the low 24 bits of word e & 3 of
 * the block at counter e >> 2, purpose P_TAIL.  Every bit is an independent Philox bit,
 * so u is uniform on [0, 2^32) like the per-site word. */
uint32_t orc_plane_uniform(uint64_t seed, uint32_t stream, uint64_t sweep, int colour, uint64_t e) {
    const int b = (int)(e & 63);
    uint32_t u = 0, out[4];
    for (int j = 0; j < 4; ++j) {
        orc_cb_block(seed, stream, sweep, colour, P_PLANES, (uint32_t)((e >> 6) * 16 + (uint64_t)j), out);
        const uint64_t p0 = (uint64_t)out[0] | ((uint64_t)out[1] << 32);
        const uint64_t p1 = (uint64_t)out[2] | ((uint64_t)out[3] << 32);
        u |= (uint32_t)((p0 >> b) & 1u) << (31 - 2 * j);
        u |= (uint32_t)((p1 >> b) & 1u) << (30 - 2 * j);
    }
    orc_cb_block(seed, stream, sweep, colour, P_TAIL, (uint32_t)(e >> 2), out);
    return u | (out[e & 3] & 0xFFFFFFu);
}

/* The Blume-Capel proposal bit of colour-class site e under bit-plane uniforms: bit e & 63
 * of plane e >> 6, where planes 2m and 2m+1 are words 0 | 1 << 32 and 2 | 3 << 32 of the
 * block at counter m, purpose P_PLANES (one block per 128 same-colour sites). */
int orc_bc_plane_bit(uint64_t seed, uint32_t stream, uint64_t sweep, int colour, uint64_t e) {
    uint32_t out[4];
    orc_cb_block(seed, stream, sweep, colour, P_PLANES, (uint32_t)(e >> 7), out);
    const uint64_t plane = (e >> 6) & 1 ? ((uint64_t)out[2] | ((uint64_t)out[3] << 32))
                                        : ((uint64_t)out[0] | ((uint64_t)out[1] << 32));
    return (int)((plane >> (e & 63)) & 1u);
}

static double u53(uint32_t hi, uint32_t lo) {
    uint64_t k = ((uint64_t)hi << 21) | (uint64_t)(lo >> 11);
    return (double)k * 0x1p-53;
}

/* ---------------------------------------------------------------------------
 * log(x) from the series log(m) = 2 atanh(s), s = (m-1)/(m+1), after splitting
 * x = 2^k m with m in [sqrt(1/2), sqrt(2)).  Plain multiplies and adds only.
 * ------------------------------------------------------------------------- */
double orc_log(double x) {
    if (x != x) return x;
    if (x < 0.0) return NAN;
    if (x == 0.0) return -INFINITY;
    if (x == INFINITY) return x;
    uint64_t b;
    memcpy(&b, &x, 8);
    int64_t k = 0;
    if ((b >> 52) == 0) { /* subnormal: scale by 2^54 */
        double y = x * 0x1p54;
        memcpy(&b, &y, 8);
        k = -54;
    }
    k += (int64_t)(b >> 52) - 1023;
    uint64_t mb = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;
    double m;
    memcpy(&m, &mb, 8);
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
    const double ln2_hi = 6.93147180369123816490e-01; /* 0x3FE62E42FEE00000 */
    const double ln2_lo = 1.90821492927058770002e-10; /* ln2 - ln2_hi */
    return kd * ln2_hi + (lm + kd * ln2_lo);
}

void orc_log_array(const double* x, double* y, int64_t n) {
    for (int64_t i = 0; i < n; ++i) y[i] = orc_log(x[i]);
}

/* logistic, src/infrastructure/utils.jl:82-88 */
static double logistic(double x) {
    if (x >= 0) return 1.0 / (1.0 + exp(-x));
    double ex = exp(x);
    return ex / (1.0 + ex);
}

static uint64_t prob_to_thr(double p) {
    if (!(p > 0.0)) return 0;
    if (p >= 1.0) return 1ull << 32;
    double v = floor(p * 4294967296.0);
    if (v >= 4294967296.0) return 1ull << 32;
    return (uint64_t)v;
}

/* Metropolis rule, src/algorithms/metropolis.jl:14-17 and
 * src/algorithms/importance_sampling.jl:80-85: accept iff lr > 0 || U < exp(lr),
 * with lr = logweight(BoltzmannEnsemble, dE) = -beta*dE (src/ensembles/boltzmann.jl:28). */
static uint64_t metropolis_thr(double beta, double dE) {
    double lr = (-beta) * dE;
    if (lr >= 0.0) return 1ull << 32;
    return prob_to_thr(exp(lr));
}

/* Glauber rule, src/algorithms/metropolis.jl:121-127: accept iff U < logistic(lr). */
static uint64_t glauber_thr(double beta, double dE) {
    double lr = (-beta) * dE;
    return prob_to_thr(logistic(lr));
}

/* Ising tables.  Entry idx = a + (2d+1)*up, a = number of neighbours aligned with the
 * site, up = (s == +1).  A flip happens iff (u ^ xmask) < thr. */
int orc_table_ising(int dim, int alg, double beta, double J, double h, uint64_t* thr,
                    uint32_t* xmask) {
    if (dim != 2 && dim != 3) return ORC_ERR_INVALID;
    int z = 2 * dim;
    for (int up = 0; up < 2; ++up) {
        for (int a = 0; a <= z; ++a) {
            int idx = a + (z + 1) * up;
            double s = up ? 1.0 : -1.0;
            double lpi = (double)(2 * a - z);            /* s_i * sum_j s_j  */
            double dpair = ((-2.0) * J) * lpi;            /* flip_changes, SpinSystems/src/ising.jl:484-489 */
            double dspin = -2.0 * s;
            double dE = (-dpair) - (h * dspin);           /* delta_energy, ising.jl:198, :491 */
            if (alg == ORC_METROPOLIS) {
                thr[idx] = metropolis_thr(beta, dE);
                xmask[idx] = 0;
            } else if (alg == ORC_GLAUBER) {
                thr[idx] = glauber_thr(beta, dE);
                xmask[idx] = 0;
            } else if (alg == ORC_HEATBATH) {
                /* ising.jl:43-58: p_plus = logistic(beta*s_old*dE), s_new = U<p_plus ? +1:-1 */
                uint64_t tp = prob_to_thr(logistic((beta * s) * dE));
                if (up) { thr[idx] = (1ull << 32) - tp; xmask[idx] = 0xFFFFFFFFu; }
                else    { thr[idx] = tp;                xmask[idx] = 0; }
            } else {
                return ORC_ERR_INVALID;
            }
        }
    }
    return ORC_OK;
}

/* _propose_state, SpinSystems/src/blume_capel.jl:21-30 */
static int bc_propose(int s_old, int b) {
    if (s_old == -1) return b ? 0 : 1;
    if (s_old == 0) return b ? -1 : 1;
    return b ? -1 : 0;
}

/* Blume-Capel tables.  Metropolis/Glauber: idx = (s_old+1)*2*(4d+1) + b*(4d+1) + (c+2d),
 * accept iff u < thr.  HeatBath: per c two cumulative thresholds (T1, T12) at
 * [2*(c+2d)], [2*(c+2d)+1]. */
int orc_table_bc(int dim, int alg, double beta, double J, double D, double h, uint64_t* thr) {
    if (dim != 2 && dim != 3) return ORC_ERR_INVALID;
    int z = 2 * dim, nc = 2 * z + 1;
    if (alg == ORC_HEATBATH) {
        for (int c = -z; c <= z; ++c) {
            /* blume_capel.jl:61-85 */
            double coupling = J * (double)c;
            double e1 = (coupling - (h * -1.0)) + D;
            double e3 = ((-coupling) - (h * 1.0)) + D;
            double w1 = exp((-beta) * e1);
            double w2 = exp((-beta) * 0.0);
            double w3 = exp((-beta) * e3);
            double zz = (w1 + w2) + w3;
            thr[2 * (c + z)] = prob_to_thr(w1 / zz);
            thr[2 * (c + z) + 1] = prob_to_thr((w1 + w2) / zz);
        }
        return ORC_OK;
    }
    if (alg != ORC_METROPOLIS && alg != ORC_GLAUBER) return ORC_ERR_INVALID;
    for (int so = -1; so <= 1; ++so)
        for (int b = 0; b < 2; ++b)
            for (int c = -z; c <= z; ++c) {
                int sn = bc_propose(so, b);
                double ds = (double)(sn - so);
                double ds2 = (double)(sn * sn - so * so);
                double dpair = ds * (J * (double)c);          /* blume_capel.jl:235-241 */
                double dE = ((-dpair) - (h * ds)) + (D * ds2); /* blume_capel.jl:247-248 */
                int idx = (so + 1) * 2 * nc + b * nc + (c + z);
                thr[idx] = alg == ORC_METROPOLIS ? metropolis_thr(beta, dE) : glauber_thr(beta, dE);
            }
    return ORC_OK;
}

/* ---------------------------------------------------------------------------
 * geometry: SpinSystems linear order (Graphs.grid vertex order, first dim fastest),
 * periodic, i = x + Lx*(y + Ly*z); colour = (x+y+z) & 1.
 * ------------------------------------------------------------------------- */
typedef struct { int dim; int64_t Lx, Ly, Lz, N; } geom_t;

static int geom_init(geom_t* g, int dim, const int32_t* L) {
    if (dim != 2 && dim != 3) return ORC_ERR_INVALID;
    g->dim = dim;
    g->Lx = L[0]; g->Ly = L[1]; g->Lz = dim == 3 ? L[2] : 1;
    for (int d = 0; d < dim; ++d)
        if (L[d] < 4 || (L[d] & 1)) return ORC_ERR_INVALID;
    g->N = g->Lx * g->Ly * g->Lz;
    return ORC_OK;
}

static inline int colour_of(const geom_t* g, int64_t i) {
    int64_t x = i % g->Lx, y = (i / g->Lx) % g->Ly, z = i / (g->Lx * g->Ly);
    return (int)((x + y + z) & 1);
}

static inline int nbr_sum(const geom_t* g, const int8_t* s, int64_t i) {
    int64_t x = i % g->Lx, y = (i / g->Lx) % g->Ly, z = i / (g->Lx * g->Ly);
    int64_t Lx = g->Lx, Ly = g->Ly, Lz = g->Lz;
    int64_t base = i - x;
    int acc = s[base + (x + 1) % Lx] + s[base + (x + Lx - 1) % Lx];
    int64_t rowbase = i - y * Lx;
    acc += s[rowbase + ((y + 1) % Ly) * Lx] + s[rowbase + ((y + Ly - 1) % Ly) * Lx];
    if (g->dim == 3) {
        int64_t plane = Lx * Ly, zb = i - z * plane;
        acc += s[zb + ((z + 1) % Lz) * plane] + s[zb + ((z + Lz - 1) % Lz) * plane];
    }
    return acc;
}

void orc_observables(const int8_t* s, int dim, const int32_t* L, int64_t* P, int64_t* M,
                     int64_t* Q) {
    geom_t g;
    if (geom_init(&g, dim, L)) { *P = *M = *Q = 0; return; }
    int64_t p = 0, m = 0, q = 0;
    for (int64_t i = 0; i < g.N; ++i) {
        int64_t x = i % g.Lx, y = (i / g.Lx) % g.Ly, z = i / (g.Lx * g.Ly);
        int si = s[i];
        int64_t xp = i - x + (x + 1) % g.Lx;
        int64_t yp = i - y * g.Lx + ((y + 1) % g.Ly) * g.Lx;
        p += si * s[xp] + si * s[yp];
        if (dim == 3) {
            int64_t pl = g.Lx * g.Ly;
            int64_t zp = i - z * pl + ((z + 1) % g.Lz) * pl;
            p += si * s[zp];
        }
        m += si;
        q += si * si;
    }
    *P = p; *M = m; *Q = q;
}

/* init!(sys, :random), SpinSystems/src/ising.jl:60-78 / SpinSystems/src/blume_capel.jl:87-109, fed by Philox */
void orc_init_random(int8_t* s, int model, int dim, const int32_t* L, uint64_t seed,
                     uint32_t stream) {
    geom_t g;
    if (geom_init(&g, dim, L)) return;
    for (int64_t i = 0; i < g.N; ++i) {
        uint32_t r = orc_site_word(seed, stream, 0, colour_of(&g, i), P_INIT, (uint64_t)i);
        if (model == ORC_ISING) s[i] = (r & 0x80000000u) ? 1 : -1;
        else s[i] = (int8_t)((int)(((uint64_t)r * 3u) >> 32) - 1);
    }
}

/* ---------------------------------------------------------------------------
 * Mode (i): checkerboard sweeps.  One sweep = colour 0 then colour 1; within a
 * colour every site sees only the other colour, so visiting the sites of one colour
 * in any order equals the simultaneous update the device performs.
 *   Ising: spin_flip!(::AbstractIsing, ::AbstractMetropolis / ::AbstractHeatBath),
 *          SpinSystems/src/ising.jl:25-58, modify! :493-498.
 *   Blume-Capel: spin_flip! blume_capel.jl:52-85, modify! :250-256.
 * ------------------------------------------------------------------------- */
static int cb_sweep(int8_t* s, int model, int dim, const int32_t* L, int alg, double beta,
                    double J, double D, double h, uint64_t seed, uint32_t stream,
                    uint64_t sweep0, int64_t nsweeps, int64_t* obs, uint64_t* attempts,
                    uint64_t* accepts, int uniforms) {
    geom_t g;
    if (geom_init(&g, dim, L)) return ORC_ERR_INVALID;
    int z = 2 * dim, nc = 2 * z + 1;
    uint64_t thr[3 * 2 * 13];
    uint32_t xm[14];
    int rc = model == ORC_ISING ? orc_table_ising(dim, alg, beta, J, h, thr, xm)
                                : orc_table_bc(dim, alg, beta, J, D, h, thr);
    if (rc) return rc;
    if (uniforms && model == ORC_ISING && L[0] % 128 != 0) return ORC_ERR_INVALID;
    const int planes = uniforms;  /* every Ising rule: flip iff (u ^ xm) < thr with the plane uniform */
    int64_t P, M, Q;
    orc_observables(s, dim, L, &P, &M, &Q);
    uint64_t att = 0, acc = 0;
    for (int64_t k = 0; k < nsweeps; ++k) {
        uint64_t t = sweep0 + (uint64_t)k;
        for (int c = 0; c < 2; ++c) {
            for (int64_t i = 0; i < g.N; ++i) {
                if (colour_of(&g, i) != c) continue;
                int so = s[i];
                int S = nbr_sum(&g, s, i);
                ++att;
                if (model == ORC_ISING) {
                    int sigma = so * S;
                    int a = (sigma + z) / 2;
                    int idx = a + (z + 1) * (so > 0);
                    /* an always-accepted class flips whatever u is */
                    uint32_t u = !planes ? orc_site_word(seed, stream, t, c, P_ACCEPT, (uint64_t)i)
                                 : thr[idx] >> 32 ? 0u : orc_plane_uniform(seed, stream, t, c, (uint64_t)i >> 1);
                    if ((uint64_t)(u ^ xm[idx]) < thr[idx]) {
                        s[i] = (int8_t)(-so);
                        P += -2 * sigma;
                        M += -2 * so;
                        ++acc;
                    }
                } else {
                    int sn;
                    if (alg == ORC_HEATBATH) {
                        uint32_t u = orc_site_word(seed, stream, t, c, P_ACCEPT, (uint64_t)i);
                        sn = (u < thr[2 * (S + z)]) ? -1 : ((u < thr[2 * (S + z) + 1]) ? 0 : 1);
                        if (sn == so) continue;
                    } else {
                        int b = planes ? orc_bc_plane_bit(seed, stream, t, c, (uint64_t)i >> 1)
                                       : (int)(orc_site_word(seed, stream, t, c, P_PROPOSE, (uint64_t)i) >> 31);
                        int idx = (so + 1) * 2 * nc + b * nc + (S + z);
                        uint32_t u = orc_site_word(seed, stream, t, c, P_ACCEPT, (uint64_t)i);
                        if (!((uint64_t)u < thr[idx])) continue;
                        sn = bc_propose(so, b);
                    }
                    int ds = sn - so;
                    s[i] = (int8_t)sn;
                    P += (int64_t)ds * S;
                    M += ds;
                    Q += sn * sn - so * so;
                    ++acc;
                }
            }
        }
        if (obs) { obs[3 * k] = P; obs[3 * k + 1] = M; obs[3 * k + 2] = Q; }
    }
    if (attempts) *attempts += att;
    if (accepts) *accepts += acc;
    return ORC_OK;
}

int orc_cb_sweep(int8_t* s, int model, int dim, const int32_t* L, int alg, double beta,
                 double J, double D, double h, uint64_t seed, uint32_t stream,
                 uint64_t sweep0, int64_t nsweeps, int64_t* obs, uint64_t* attempts,
                 uint64_t* accepts) {
    return cb_sweep(s, model, dim, L, alg, beta, J, D, h, seed, stream, sweep0, nsweeps, obs, attempts, accepts, 0);
}

/* The same sweeps with the uniforms form `uniforms` (0 per-site words, 1 bit planes: every
 * Ising rule, Ising lattices with Lx a multiple of 128; the Blume-Capel proposal bits). */
int orc_cb_sweep_u(int8_t* s, int model, int dim, const int32_t* L, int alg, double beta,
                   double J, double D, double h, uint64_t seed, uint32_t stream,
                   uint64_t sweep0, int64_t nsweeps, int64_t* obs, uint64_t* attempts,
                   uint64_t* accepts, int uniforms) {
    return cb_sweep(s, model, dim, L, alg, beta, J, D, h, seed, stream, sweep0, nsweeps, obs, attempts, accepts,
                    uniforms);
}

/* ---------------------------------------------------------------------------
 * Mode (ii): the reference's sequential random-site order with FP64 decisions.
 *   pick_site:   SpinSystems/src/abstractions.jl:19 (rand(rng, UInt) % N + 1)
 *   Metropolis:  SpinSystems/src/ising.jl:35-41 -> src/algorithms/metropolis.jl:14-17 ->
 *                src/algorithms/importance_sampling.jl:80-85
 *   Glauber:     src/algorithms/metropolis.jl:121-127
 *   HeatBath:    SpinSystems/src/ising.jl:43-58, SpinSystems/src/blume_capel.jl:61-85
 *   BC proposal: blume_capel.jl:21-30, 52-59
 * Attempt a draws Philox(seed, (a lo, a hi, P_SEQ<<24, stream)) -> site from words
 * 0,1 and U from words 2,3; Blume-Capel proposals take the top bit of word 0 of
 * Philox(seed, (a lo, a hi, P_SEQ2<<24, stream)).
 * ------------------------------------------------------------------------- */
int orc_seq_attempts(int8_t* s, int model, int dim, const int32_t* L, int alg, double beta,
                     double J, double D, double h, uint64_t seed, uint32_t stream,
                     uint64_t attempt0, int64_t nattempts, uint64_t* steps,
                     uint64_t* accepted) {
    geom_t g;
    if (geom_init(&g, dim, L)) return ORC_ERR_INVALID;
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint64_t st = 0, ac = 0;
    for (int64_t k = 0; k < nattempts; ++k) {
        uint64_t a = attempt0 + (uint64_t)k;
        uint32_t ctr[4] = {(uint32_t)a, (uint32_t)(a >> 32), (uint32_t)P_SEQ << 24, stream};
        uint32_t w[4];
        orc_philox4x32_10(ctr, key, w);
        int64_t i = (int64_t)((((uint64_t)w[0] << 32) | w[1]) % (uint64_t)g.N);
        double U = u53(w[2], w[3]);
        int so = s[i];
        int S = nbr_sum(&g, s, i);
        ++st;
        if (model == ORC_ISING) {
            double lpi = (double)(so * S);
            double dpair = ((-2.0) * J) * lpi;
            double dspin = -2.0 * so;
            double dE = (-dpair) - (h * dspin);
            int flip;
            if (alg == ORC_METROPOLIS) {
                double lr = (-beta) * dE;
                flip = (lr > 0) || (U < exp(lr));
            } else if (alg == ORC_GLAUBER) {
                double lr = (-beta) * dE;
                flip = U < logistic(lr);
            } else {
                double pp = logistic((beta * (double)so) * dE);
                int sn = U < pp ? 1 : -1;
                flip = sn != so;
            }
            if (flip) { s[i] = (int8_t)(-so); ++ac; }
        } else {
            int sn;
            if (alg == ORC_HEATBATH) {
                double coupling = J * (double)S;
                double e1 = (coupling - (h * -1.0)) + D;
                double e3 = ((-coupling) - (h * 1.0)) + D;
                double w1 = exp((-beta) * e1), w2 = exp((-beta) * 0.0), w3 = exp((-beta) * e3);
                double zz = (w1 + w2) + w3;
                double r = U * zz;
                sn = r < w1 ? -1 : (r < (w1 + w2) ? 0 : 1);
                if (sn != so) { s[i] = (int8_t)sn; ++ac; }
            } else {
                uint32_t c2[4] = {(uint32_t)a, (uint32_t)(a >> 32), (uint32_t)P_SEQ2 << 24, stream};
                uint32_t w2[4];
                orc_philox4x32_10(c2, key, w2);
                int b = (int)(w2[0] >> 31);
                sn = bc_propose(so, b);
                double ds = (double)(sn - so), ds2 = (double)(sn * sn - so * so);
                double dE = ((-(ds * (J * (double)S))) - (h * ds)) + (D * ds2);
                double lr = (-beta) * dE;
                int acc = alg == ORC_METROPOLIS ? ((lr > 0) || (U < exp(lr))) : (U < logistic(lr));
                if (acc) { s[i] = (int8_t)sn; ++ac; }
            }
        }
    }
    if (steps) *steps += st;
    if (accepted) *accepted += ac;
    return ORC_OK;
}

/* ---------------------------------------------------------------------------
 * Flat-histogram sweeps in checkerboard order.
 *   generic importance-sampling spin flip: SpinSystems/src/ising.jl:25-33,
 *                                SpinSystems/src/blume_capel.jl:41-50
 *   accept!(alg, x_new, x_old):  src/algorithms/importance_sampling.jl:69-85
 *   MUCA record_visit!:          src/ensembles/multicanonical.jl:25-30 (h[x] += 1)
 *   WangLandau accept!:          src/algorithms/wang_landau.jl:29-37 (lw[x_vis] -= logf)
 *   BinnedObject integer index:  src/infrastructure/binned_object.jl:22-24 (div(x-start,step)+1)
 * The decision lr > 0 || U < exp(lr) is evaluated as lr > 0 || log(U) < lr.  An
 * energy outside the bins stops the run before the attempt is counted (the
 * reference throws BoundsError from lw(x_new) with the counters unchanged,
 * test/test_multicanonical.jl:39-43).  Energies must be integers: J, D, h integral.
 * The Wang-Landau run also counts visits in H (for the flatness test).
 * ------------------------------------------------------------------------- */
static int bin_of(int64_t E, int64_t start, int64_t step, int64_t nbins, int64_t* b) {
    int64_t q = (E - start) / step; /* truncating, as Julia div */
    if (q < 0 || q >= nbins) return 0;
    *b = q;
    return 1;
}

static int flathist_run(int8_t* s, int model, int dim, const int32_t* L, double J, double D,
                        double h, int mode, double* lnw, int64_t* H, int64_t start,
                        int64_t step, int64_t nbins, double logf, uint64_t seed,
                        uint32_t stream, uint64_t sweep0, int64_t nsweeps, int64_t* obs,
                        uint64_t* steps, uint64_t* accepted, double* tr_u, double* tr_lr,
                        int64_t tr_cap, int64_t* tr_n) {
    geom_t g;
    if (geom_init(&g, dim, L)) return ORC_ERR_INVALID;
    if (step <= 0 || nbins <= 0) return ORC_ERR_INVALID;
    int64_t Ji = (int64_t)J, Di = (int64_t)D, hi = (int64_t)h;
    if ((double)Ji != J || (double)Di != D || (double)hi != h) return ORC_ERR_INVALID;
    int64_t P, M, Q;
    orc_observables(s, dim, L, &P, &M, &Q);
    int64_t E = -Ji * P + Di * Q - hi * M;
    int64_t bo;
    if (!bin_of(E, start, step, nbins, &bo)) return ORC_ERR_RANGE;
    uint64_t st = 0, ac = 0;
    int rc = ORC_OK;
    for (int64_t k = 0; k < nsweeps && rc == ORC_OK; ++k) {
        uint64_t t = sweep0 + (uint64_t)k;
        for (int c = 0; c < 2 && rc == ORC_OK; ++c) {
            for (int64_t i = 0; i < g.N; ++i) {
                if (colour_of(&g, i) != c) continue;
                int so = s[i];
                int S = nbr_sum(&g, s, i);
                int sn;
                if (model == ORC_ISING) sn = -so;
                else sn = bc_propose(so, (int)(orc_site_word(seed, stream, t, c, P_PROPOSE, (uint64_t)i) >> 31));
                int64_t ds = sn - so, dq = sn * sn - so * so, dp = ds * S;
                int64_t dE = -Ji * dp + Di * dq - hi * ds;
                int64_t En = E + dE, bn;
                if (!bin_of(En, start, step, nbins, &bn)) { rc = ORC_ERR_RANGE; break; }
                double lr = lnw[bn] - lnw[bo];
                double U = u53(orc_site_word(seed, stream, t, c, P_ACCEPT, (uint64_t)i),
                               orc_site_word(seed, stream, t, c, P_LOW, (uint64_t)i));
                int acc = (lr > 0) || (orc_log(U) < lr);
                if (tr_n && *tr_n < tr_cap) {
                    tr_u[*tr_n] = U;
                    tr_lr[*tr_n] = lr;
                    ++*tr_n;
                }
                ++st;
                if (acc) {
                    ++ac;
                    s[i] = (int8_t)sn;
                    P += dp; M += ds; Q += dq;
                    E = En;
                    bo = bn;
                }
                if (mode == ORC_WL) lnw[bo] -= logf;
                H[bo] += 1;
            }
        }
        if (rc == ORC_OK && obs) { obs[3 * k] = P; obs[3 * k + 1] = M; obs[3 * k + 2] = Q; }
    }
    if (steps) *steps += st;
    if (accepted) *accepted += ac;
    return rc;
}

int orc_flathist_sweep(int8_t* s, int model, int dim, const int32_t* L, double J, double D,
                       double h, int mode, double* lnw, int64_t* H, int64_t start,
                       int64_t step, int64_t nbins, double logf, uint64_t seed,
                       uint32_t stream, uint64_t sweep0, int64_t nsweeps, int64_t* obs,
                       uint64_t* steps, uint64_t* accepted) {
    return flathist_run(s, model, dim, L, J, D, h, mode, lnw, H, start, step, nbins, logf, seed, stream,
                        sweep0, nsweeps, obs, steps, accepted, NULL, NULL, 0, NULL);
}

/* The same sweeps, also recording the (U, lr) of every decision, in order (up to tr_cap). */
int orc_flathist_trace(int8_t* s, int model, int dim, const int32_t* L, double J, double D,
                       double h, int mode, double* lnw, int64_t* H, int64_t start,
                       int64_t step, int64_t nbins, double logf, uint64_t seed,
                       uint32_t stream, uint64_t sweep0, int64_t nsweeps, double* tr_u,
                       double* tr_lr, int64_t tr_cap, int64_t* tr_n) {
    uint64_t st = 0, ac = 0;
    *tr_n = 0;
    return flathist_run(s, model, dim, L, J, D, h, mode, lnw, H, start, step, nbins, logf, seed, stream,
                        sweep0, nsweeps, NULL, &st, &ac, tr_u, tr_lr, tr_cap, tr_n);
}

/* update!(::MulticanonicalEnsemble; mode=:simple), src/ensembles/multicanonical.jl:32-43 */
void orc_muca_update(double* lnw, const int64_t* H, int64_t nbins) {
    for (int64_t b = 0; b < nbins; ++b) {
        double logh = H[b] > 0 ? orc_log((double)H[b]) : 0.0;
        lnw[b] -= logh;
    }
}

/* Wang-Landau flatness (Wang & Landau, PRL 86, 2050 (2001)): over the bins visited
 * at least once in the run, min H >= flatness * mean H. */
int orc_wl_flat(const int64_t* H, const uint8_t* visited, int64_t nbins, double flatness,
                double* ratio) {
    int64_t mn = INT64_MAX, sum = 0, cnt = 0;
    for (int64_t b = 0; b < nbins; ++b) {
        if (!visited[b]) continue;
        if (H[b] < mn) mn = H[b];
        sum += H[b];
        ++cnt;
    }
    if (cnt == 0 || sum == 0) { if (ratio) *ratio = 0.0; return 0; }
    double mean = (double)sum / (double)cnt;
    double r = (double)mn / mean;
    if (ratio) *ratio = r;
    return r >= flatness;
}

/* ---------------------------------------------------------------------------
 * Replica exchange, src/algorithms/replica_exchange.jl:110-178 (threads update!):
 * even/odd neighbour pairs by stage, lr = exchange_log_ratio, accept iff
 * lr > 0 || U < exp(lr) (evaluated as log(U) < lr), swap the ladder positions.
 * pos[r] = 0-based ladder position held by replica r (the reference's indices - 1).
 * U for pair p after sweep t: Philox(seed, (p, t lo, t hi16 | P_EXCHANGE<<24, ladder))
 * words 0 and 1.
 * ------------------------------------------------------------------------- */
int orc_pt_exchange(int n, const double* betas, int32_t* pos, int32_t* stage,
                    const double* x, uint64_t seed, uint32_t ladder, uint64_t t,
                    uint64_t* steps, uint64_t* accepted) {
    if (n < 2) return ORC_ERR_INVALID;
    int32_t* rep = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    for (int r = 0; r < n; ++r) rep[pos[r]] = r;
    int first = (*stage % 2 == 0) ? 0 : 1;
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int p = first; p < n - 1; p += 2) {
        int ri = rep[p], rj = rep[p + 1];
        steps[p] += 1;
        uint32_t ctr[4] = {(uint32_t)p, (uint32_t)t,
                           ((uint32_t)(t >> 32) & 0xFFFFu) | ((uint32_t)P_EXCHANGE << 24), ladder};
        uint32_t w[4];
        orc_philox4x32_10(ctr, key, w);
        double U = u53(w[0], w[1]);
        double bi = betas[p], bj = betas[p + 1];
        double xi = x[ri], xj = x[rj];
        double lr = (((-bi) * xj) - ((-bi) * xi)) + (((-bj) * xi) - ((-bj) * xj));
        if ((lr > 0) || (orc_log(U) < lr)) {
            accepted[p] += 1;
            pos[ri] = p + 1;
            pos[rj] = p;
        }
    }
    *stage = 1 - *stage;
    free(rep);
    return ORC_OK;
}

/* ---------------------------------------------------------------------------
 * CPU baseline harness: one independent chain per thread (the reference's
 * ParallelChains threads pattern, src/infrastructure/parallel_chains.jl:99-105).
 * ------------------------------------------------------------------------- */
typedef struct {
    int model, dim, alg;
    int32_t L[3];
    double beta, J, D, h;
    uint64_t seed;
    uint32_t stream;
    int64_t attempts;
    int8_t* s;
    int rc;
} bench_arg_t;

static void* bench_init_thread(void* p) {
    bench_arg_t* a = (bench_arg_t*)p;
    orc_init_random(a->s, a->model, a->dim, a->L, a->seed, a->stream);
    return NULL;
}

static void* bench_thread(void* p) {
    bench_arg_t* a = (bench_arg_t*)p;
    uint64_t st = 0, ac = 0;
    a->rc = orc_seq_attempts(a->s, a->model, a->dim, a->L, a->alg, a->beta, a->J, a->D, a->h,
                             a->seed, a->stream, 0, a->attempts, &st, &ac);
    return NULL;
}

int orc_bench_seq(int model, int dim, const int32_t* L, int alg, double beta, double J,
                  double D, double h, uint64_t seed, int nthreads, int64_t attempts_per_thread,
                  double* seconds) {
    geom_t g;
    if (geom_init(&g, dim, L) || nthreads < 1) return ORC_ERR_INVALID;
    bench_arg_t* args = (bench_arg_t*)calloc((size_t)nthreads, sizeof(bench_arg_t));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int k = 0; k < nthreads; ++k) {
        bench_arg_t* a = &args[k];
        a->model = model; a->dim = dim; a->alg = alg;
        a->L[0] = L[0]; a->L[1] = L[1]; a->L[2] = dim == 3 ? L[2] : 1;
        a->beta = beta; a->J = J; a->D = D; a->h = h;
        a->seed = seed; a->stream = (uint32_t)k; a->attempts = attempts_per_thread;
        a->s = (int8_t*)malloc((size_t)g.N);
    }
    /* every chain's start from its own stream, one thread each, before the clock starts */
    for (int k = 0; k < nthreads; ++k) pthread_create(&th[k], NULL, bench_init_thread, &args[k]);
    for (int k = 0; k < nthreads; ++k) pthread_join(th[k], NULL);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int k = 0; k < nthreads; ++k) pthread_create(&th[k], NULL, bench_thread, &args[k]);
    int rc = ORC_OK;
    for (int k = 0; k < nthreads; ++k) {
        pthread_join(th[k], NULL);
        if (args[k].rc) rc = args[k].rc;
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    *seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
    for (int k = 0; k < nthreads; ++k) free(args[k].s);
    free(args);
    free(th);
    return rc;
}

/* ---------------------------------------------------------------------------
 * General graphs and couplings: IsingGraph (one J over a neighbour list,
 * SpinSystems/src/ising.jl:86-139) and IsingMatrix (symmetric sparse J_ij,
 * ising.jl:221-292), each with no field, a uniform field or a field per site.
 * ------------------------------------------------------------------------- */

/* exp(x): Cody & Waite argument reduction x = k ln2 + r, |r| <= ln2/2, with ln2 split
 * into a 32-bit head (k * head exact) and a tail; exp(r) from its Taylor series up to
 * r^13/13! in Horner form; then the exponent of 2^k is put in with one or two exact
 * scalings.  Plain multiplies and adds only, so every machine gives the same bits. */
double orc_exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.2) return 0.0;
    double kd = floor(x * 0x1.71547652b82fep+0 + 0.5);
    double r = (x - kd * 0x1.62e42fee00000p-1) - kd * 0x1.a39ef35793c76p-33;
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
    int k = (int)kd;
    if (k > 1023) return (p * ldexp(1.0, k - 1)) * 2.0;
    if (k < -1021) return (p * ldexp(1.0, k + 64)) * 0x1p-64;
    return p * ldexp(1.0, k);
}

/* logistic(x), src/infrastructure/utils.jl:82-88, on orc_exp */
double orc_logistic(double x) {
    if (x >= 0) return 1.0 / (1.0 + orc_exp(-x));
    double ex = orc_exp(x);
    return ex / (1.0 + ex);
}

/* First-fit colouring in vertex order: a vertex takes the smallest colour that none of
 * its lower-numbered neighbours holds.  Diagonal entries are not neighbours.  Returns
 * the number of colours. */
int orc_graph_colour(int64_t n, const int64_t* rowptr, const int32_t* col, int32_t* colour) {
    int64_t maxdeg = 0;
    for (int64_t v = 0; v < n; ++v)
        if (rowptr[v + 1] - rowptr[v] > maxdeg) maxdeg = rowptr[v + 1] - rowptr[v];
    int64_t* seen = (int64_t*)malloc((size_t)(maxdeg + 2) * sizeof(int64_t));
    for (int64_t c = 0; c < maxdeg + 2; ++c) seen[c] = -1;
    int ncol = 0;
    for (int64_t v = 0; v < n; ++v) {
        for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e) {
            int64_t u = col[e];
            if (u < v) seen[colour[u]] = v;
        }
        int c = 0;
        while (seen[c] == v) ++c;
        colour[v] = c;
        if (c + 1 > ncol) ncol = c + 1;
    }
    free(seen);
    return ncol;
}

/* init!(sys, :random) for a graph: site v takes the top bit of word v&3 of the Philox
 * block (v>>2, 0, 8<<24, stream). */
void orc_graph_init_random(int8_t* s, int64_t n, uint64_t seed, uint32_t stream) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int64_t v = 0; v < n; ++v) {
        uint32_t ctr[4] = {(uint32_t)(v >> 2), 0u, 8u << 24, stream}, out[4];
        orc_philox4x32_10(ctr, key, out);
        s[v] = (out[v & 3] & 0x80000000u) ? 1 : -1;
    }
}

/* local_pair_interactions: SpinSystems/src/abstractions.jl:41-48 (integer sum over the neighbour list)
 * and ising.jl:294-304 (FP64 sum of s_i J_ij s_j over the stored entries, j != i). */
static double graph_dpair(const int8_t* s, int64_t v, const int64_t* rowptr, const int32_t* col,
                          const double* Jv, double J) {
    int si = s[v];
    if (Jv) {
        double acc = 0.0;
        for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e) {
            if (col[e] == v) continue;
            acc += ((double)si * Jv[e]) * (double)s[col[e]];
        }
        return -2.0 * acc;  /* flip_changes, ising.jl:351-356 */
    }
    int64_t lpi = 0;
    for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e)
        if (col[e] != v) lpi += si * s[col[e]];
    return (-2.0 * J) * (double)lpi;  /* flip_changes, ising.jl:187-191 */
}

/* delta_energy, ising.jl:198 and :362: -Δpair - h Δspin */
static double graph_delta_energy(const int8_t* s, int64_t v, const int64_t* rowptr,
                                 const int32_t* col, const double* Jv, double J,
                                 const double* hv, double h) {
    double dpair = graph_dpair(s, v, rowptr, col, Jv, J);
    double dspin = (double)(-2 * s[v]);
    if (hv) return -dpair - hv[v] * dspin;
    if (h != 0.0) return -dpair - h * dspin;
    return -dpair;
}

double orc_graph_delta_energy(const int8_t* s, int64_t v, const int64_t* rowptr,
                              const int32_t* col, const double* Jv, double J, const double* hv,
                              double h) {
    return graph_delta_energy(s, v, rowptr, col, Jv, J, hv, h);
}

/* _full_energy and magnetization, ising.jl:161-185 and :306-322: -pair - field */
void orc_graph_observables(const int8_t* s, int64_t n, const int64_t* rowptr, const int32_t* col,
                           const double* Jv, double J, const double* hv, double h, double* E,
                           int64_t* M) {
    double pair;
    if (Jv) {
        double acc = 0.0;
        for (int64_t v = 0; v < n; ++v) acc += -0.5 * graph_dpair(s, v, rowptr, col, Jv, J);
        pair = acc / 2;
    } else {
        int64_t acc = 0;
        for (int64_t v = 0; v < n; ++v)
            for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e)
                if (col[e] != v) acc += s[v] * s[col[e]];
        pair = J * (double)(acc / 2);
    }
    int64_t m = 0;
    double field = 0.0;
    for (int64_t v = 0; v < n; ++v) {
        m += s[v];
        if (hv) field += hv[v] * (double)s[v];
    }
    if (!hv) field = h * (double)m;
    *E = -pair - field;
    *M = m;
}

/* Colour-class sweeps.  Sweep t visits colour 0, 1, ... in turn and, inside a colour, the
 * sites in increasing order.  The l-th site of class c takes its 53-bit uniform from words
 * 2b and 2b+1, b = (l>>5)&1, of the Philox block (B, t lo, t hi16 | 7<<24, stream) with
 * B = B_c + 32 (l>>6) + (l&31), where B_c = sum over earlier classes of 32 ceil(n_c'/64):
 * one block serves the sites l and l+32 of a 64-site group.  Sites of one colour share no
 * edge, so any order inside a colour gives the same result.
 *   Metropolis: accept!(alg, ΔE), metropolis.jl:14-17 with _accept!,
 *               importance_sampling.jl:80-85: lr = -β ΔE; lr > 0 or u < exp(lr).
 *   Glauber:    metropolis.jl:121-127: u < logistic(lr).
 *   HeatBath:   spin_flip!(::AbstractIsing, ::AbstractHeatBath), ising.jl:43-58:
 *               p_plus = logistic(β s_old ΔE); s_new = u < p_plus ? +1 : -1.
 * E and M are the cached observables, updated by modify! (ising.jl:200-218, :364-377).
 * E_series / M_series (may be NULL) get the values after each sweep. */
int orc_graph_sweep(int8_t* s, int64_t n, const int64_t* rowptr, const int32_t* col,
                    const double* Jv, double J, const double* hv, double h, int alg, double beta,
                    uint64_t seed, uint32_t stream, uint64_t sweep0, int64_t nsweeps, double* E,
                    int64_t* M, double* E_series, int64_t* M_series, uint64_t* attempts,
                    uint64_t* accepts) {
    if (alg < ORC_METROPOLIS || alg > ORC_HEATBATH || n < 1) return ORC_ERR_INVALID;
    int32_t* colour = (int32_t*)malloc((size_t)n * sizeof(int32_t));
    int ncol = orc_graph_colour(n, rowptr, col, colour);
    int64_t* order = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    uint64_t* block = (uint64_t*)malloc((size_t)n * sizeof(uint64_t));
    int* word = (int*)malloc((size_t)n * sizeof(int));
    int64_t q = 0;
    uint64_t B_c = 0;
    for (int c = 0; c < ncol; ++c) {
        int64_t l = 0;
        for (int64_t v = 0; v < n; ++v)
            if (colour[v] == c) {
                order[q] = v;
                block[q] = B_c + 32 * (uint64_t)(l >> 6) + (uint64_t)(l & 31);
                word[q] = 2 * (int)((l >> 5) & 1);
                ++q;
                ++l;
            }
        B_c += 32 * (uint64_t)((l + 63) / 64);
    }
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint64_t acc_n = 0;
    for (int64_t t = 0; t < nsweeps; ++t) {
        uint64_t sw = sweep0 + (uint64_t)t;
        for (q = 0; q < n; ++q) {
            int64_t v = order[q];
            uint32_t ctr[4] = {(uint32_t)block[q], (uint32_t)sw,
                               ((uint32_t)(sw >> 32) & 0xFFFFu) | (7u << 24), stream}, out[4];
            orc_philox4x32_10(ctr, key, out);
            double u = u53(out[word[q]], out[word[q] + 1]);
            int so = s[v];
            double dE = graph_delta_energy(s, v, rowptr, col, Jv, J, hv, h);
            int flip;
            if (alg == ORC_METROPOLIS) {
                double lr = -beta * dE;
                flip = (lr > 0) || (u < orc_exp(lr));
            } else if (alg == ORC_GLAUBER) {
                flip = u < orc_logistic(-beta * dE);
            } else {
                int up = u < orc_logistic((beta * (double)so) * dE);
                flip = up != (so == 1);
            }
            if (flip) {
                s[v] = (int8_t)(-so);
                *E += dE;
                *M += -2 * so;
                ++acc_n;
            }
        }
        if (E_series) E_series[t] = *E;
        if (M_series) M_series[t] = *M;
    }
    *attempts += (uint64_t)n * (uint64_t)nsweeps;
    *accepts += acc_n;
    free(word);
    free(block);
    free(order);
    free(colour);
    return ORC_OK;
}

/* ---------------------------------------------------------------------------
 * integrated_autocorrelation_time(samples; max_lag, c), src/measurements/
 * autocorrelations.jl:28-67: tau = 1/2 + sum_t C(t) with C(t) the normalised
 * autocovariance at lag t (cov over the n - t overlapping pairs), truncated at the
 * first non-positive C(t) or when t > c * tau.  max_lag <= 0 means floor(n/2).
 * Returns -1 for invalid arguments (the reference's ArgumentError).
 * ------------------------------------------------------------------------- */
double orc_tau_int(const double* x, int64_t n, int64_t max_lag, double c) {
    if (n < 2 || !(c > 0)) return -1.0;
    int64_t cap = n / 2;
    if (max_lag > 0) {
        if (max_lag > cap) return -1.0;
        cap = max_lag;
    }
    double mu = 0.0;
    for (int64_t i = 0; i < n; ++i) mu += x[i];
    mu = mu / (double)n;
    double* ce = (double*)malloc((size_t)n * sizeof(double));
    double c0 = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        ce[i] = x[i] - mu;
        c0 += ce[i] * ce[i];
    }
    c0 = c0 / (double)n;
    double tau = 0.5;
    if (c0 > 0) {
        for (int64_t lag = 1; lag <= cap; ++lag) {
            double cov = 0.0;
            for (int64_t i = 0; i < n - lag; ++i) cov += ce[i] * ce[i + lag];
            cov = cov / (double)(n - lag);
            double C = cov / c0;
            if (C <= 0) break;
            double next = tau + C;
            if ((double)lag > c * next) break;
            tau = next;
        }
    }
    free(ce);
    return tau > 0.5 ? tau : 0.5;
}

/* ---------------------------------------------------------------------------
 * Blume-Capel on general graphs: BlumeCapelGraph (one J, blume_capel.jl:117-276) and
 * BlumeCapelMatrix (symmetric sparse J_ij, :278-466), no / uniform / per-site field.
 * Spins in {-1, 0, 1}; Jv NULL means one coupling J.
 * ------------------------------------------------------------------------- */

/* local_coupling: J * sum_j s_j (:227-229) or the FP64 sum of J_ij s_j over the row,
 * diagonal skipped (:368-377) */
static double bcg_coupling(const int8_t* s, int64_t v, const int64_t* rowptr, const int32_t* col,
                           const double* Jv, double J) {
    if (Jv) {
        double acc = 0.0;
        for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e)
            if (col[e] != v) acc += Jv[e] * (double)s[col[e]];
        return acc;
    }
    int64_t sum = 0;
    for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e)
        if (col[e] != v) sum += s[col[e]];
    return J * (double)sum;
}

static double bcg_field(int64_t v, const double* hv, double h) { return hv ? hv[v] : h; }

/* delta_energy(sys, i, s_new), :36-39 with propose_changes :235-241 / :423-429 and :247-248:
 * -Δspin*c - h Δspin + D Δspin2 */
double orc_bcg_delta_energy(const int8_t* s, int64_t v, int s_new, const int64_t* rowptr,
                            const int32_t* col, const double* Jv, double J, double D,
                            const double* hv, double h) {
    int so = s[v];
    int ds = s_new - so, ds2 = s_new * s_new - so * so;
    double dpair = (double)ds * bcg_coupling(s, v, rowptr, col, Jv, J);
    double dfield = (hv || h != 0.0) ? bcg_field(v, hv, h) * (double)ds : 0.0;
    return (-dpair - dfield) + D * (double)ds2;
}

/* _full_energy (:225, :417) and sum(spins) */
void orc_bcg_observables(const int8_t* s, int64_t n, const int64_t* rowptr, const int32_t* col,
                         const double* Jv, double J, double D, const double* hv, double h,
                         double* E, int64_t* M) {
    double pair;
    if (Jv) {
        double acc = 0.0;
        for (int64_t v = 0; v < n; ++v) {
            double a = 0.0;
            for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e)
                if (col[e] != v) a += ((double)s[v] * Jv[e]) * (double)s[col[e]];
            acc += a;
        }
        pair = acc / 2;
    } else {
        double pu = 0.0;
        for (int64_t v = 0; v < n; ++v) {
            int64_t a = 0;
            for (int64_t e = rowptr[v]; e < rowptr[v + 1]; ++e)
                if (col[e] != v) a += s[v] * s[col[e]];
            pu += (double)a;
        }
        pair = J * (pu / 2);
    }
    int64_t m = 0, q = 0;
    double field = 0.0;
    for (int64_t v = 0; v < n; ++v) {
        m += s[v];
        q += s[v] * s[v];
        if (hv) field += hv[v] * (double)s[v];
    }
    if (!hv) field = h * (double)m;
    *E = (-pair - field) + D * (double)q;
    *M = m;
}

/* init!(sys, :random) of a graph: state floor(3 w / 2^32) - 1 from word v&3 of block
 * (v>>2, 0, 8<<24, stream) */
void orc_bcg_init_random(int8_t* s, int64_t n, uint64_t seed, uint32_t stream) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int64_t v = 0; v < n; ++v) {
        uint32_t ctr[4] = {(uint32_t)(v >> 2), 0u, 8u << 24, stream}, out[4];
        orc_philox4x32_10(ctr, key, out);
        s[v] = (int8_t)((int)(((uint64_t)out[v & 3] * 3u) >> 32) - 1);
    }
}

/* Colour-class sweeps (the order and uniforms of orc_graph_sweep); the proposal of
 * Metropolis / Glauber is bit 0 of the low word of the site's uniform (a bit the 53-bit
 * uniform does not use), standing in for rand(rng, Bool) of _propose_state (:21-30).
 *   Metropolis / Glauber: spin_flip! :52-59 (accept!(alg, ΔE)).
 *   HeatBath: :61-85 -- three Boltzmann weights, r = u z, cumulative choice. */
int orc_bcg_sweep(int8_t* s, int64_t n, const int64_t* rowptr, const int32_t* col,
                  const double* Jv, double J, double D, const double* hv, double h, int alg,
                  double beta, uint64_t seed, uint32_t stream, uint64_t sweep0, int64_t nsweeps,
                  double* E, int64_t* M, double* E_series, int64_t* M_series, uint64_t* attempts,
                  uint64_t* accepts) {
    if (alg < ORC_METROPOLIS || alg > ORC_HEATBATH || n < 1) return ORC_ERR_INVALID;
    int32_t* colour = (int32_t*)malloc((size_t)n * sizeof(int32_t));
    int ncol = orc_graph_colour(n, rowptr, col, colour);
    int64_t* order = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    uint64_t* block = (uint64_t*)malloc((size_t)n * sizeof(uint64_t));
    int* word = (int*)malloc((size_t)n * sizeof(int));
    int64_t q = 0;
    uint64_t B_c = 0;
    for (int c = 0; c < ncol; ++c) {
        int64_t l = 0;
        for (int64_t v = 0; v < n; ++v)
            if (colour[v] == c) {
                order[q] = v;
                block[q] = B_c + 32 * (uint64_t)(l >> 6) + (uint64_t)(l & 31);
                word[q] = 2 * (int)((l >> 5) & 1);
                ++q;
                ++l;
            }
        B_c += 32 * (uint64_t)((l + 63) / 64);
    }
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint64_t acc_n = 0;
    for (int64_t t = 0; t < nsweeps; ++t) {
        uint64_t sw = sweep0 + (uint64_t)t;
        for (q = 0; q < n; ++q) {
            int64_t v = order[q];
            uint32_t ctr[4] = {(uint32_t)block[q], (uint32_t)sw,
                               ((uint32_t)(sw >> 32) & 0xFFFFu) | (7u << 24), stream}, out[4];
            orc_philox4x32_10(ctr, key, out);
            uint32_t hi = out[word[q]], lo = out[word[q] + 1];
            double u = u53(hi, lo);
            int so = s[v], sn;
            if (alg == ORC_HEATBATH) {
                double c = bcg_coupling(s, v, rowptr, col, Jv, J);
                double hi_ = (hv || h != 0.0) ? bcg_field(v, hv, h) : 0.0;
                double e1 = (c - hi_ * (-1.0)) + D;
                double e3 = (-c - hi_) + D;
                double w1 = orc_exp(-beta * e1), w2 = orc_exp(-beta * 0.0), w3 = orc_exp(-beta * e3);
                double z = (w1 + w2) + w3;
                double r = u * z;
                sn = r < w1 ? -1 : (r < w1 + w2 ? 0 : 1);
            } else {
                sn = bc_propose(so, (int)(lo & 1u));
                double dE = orc_bcg_delta_energy(s, v, sn, rowptr, col, Jv, J, D, hv, h);
                double lr = -beta * dE;
                int acc = alg == ORC_METROPOLIS ? ((lr > 0) || (u < orc_exp(lr))) : (u < orc_logistic(lr));
                if (!acc) sn = so;
            }
            if (sn != so) {
                double dE = orc_bcg_delta_energy(s, v, sn, rowptr, col, Jv, J, D, hv, h);
                s[v] = (int8_t)sn;
                *E += dE;
                *M += sn - so;
                ++acc_n;
            }
        }
        if (E_series) E_series[t] = *E;
        if (M_series) M_series[t] = *M;
    }
    *attempts += (uint64_t)n * (uint64_t)nsweeps;
    *accepts += acc_n;
    free(word);
    free(block);
    free(order);
    free(colour);
    return ORC_OK;
}

/* The reference's own order on a general graph: nattempts x spin_flip!(sys, alg) at a
 * uniformly random vertex (pick_site, SpinSystems/src/abstractions.jl:19) with the site
 * rules of orc_graph_sweep / orc_bcg_sweep.  Attempt a draws Philox(seed, (a lo, a hi,
 * P_SEQ<<24, stream)): vertex ((w0<<32)|w1) mod n, u = u53(w2, w3); a Blume-Capel
 * Metropolis / Glauber proposal is the top bit of word 0 of (a lo, a hi, P_SEQ2<<24,
 * stream).  bc selects the Blume-Capel rules (crystal field D).  E and M are the cached
 * observables, updated after each accepted move. */
int orc_graph_seq_attempts(int8_t* s, int64_t n, const int64_t* rowptr, const int32_t* col,
                           const double* Jv, double J, const double* hv, double h, int bc, double D,
                           int alg, double beta, uint64_t seed, uint32_t stream, uint64_t attempt0,
                           int64_t nattempts, double* E, int64_t* M, uint64_t* attempts,
                           uint64_t* accepts) {
    if (alg < ORC_METROPOLIS || alg > ORC_HEATBATH || n < 1) return ORC_ERR_INVALID;
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint64_t acc_n = 0;
    for (int64_t k = 0; k < nattempts; ++k) {
        uint64_t a = attempt0 + (uint64_t)k;
        uint32_t ctr[4] = {(uint32_t)a, (uint32_t)(a >> 32), (uint32_t)P_SEQ << 24, stream}, w[4];
        orc_philox4x32_10(ctr, key, w);
        int64_t v = (int64_t)((((uint64_t)w[0] << 32) | w[1]) % (uint64_t)n);
        double u = u53(w[2], w[3]);
        int so = s[v], sn = so;
        double dE = 0.0;
        if (!bc) {
            dE = graph_delta_energy(s, v, rowptr, col, Jv, J, hv, h);
            int flip;
            if (alg == ORC_METROPOLIS) {
                double lr = -beta * dE;
                flip = (lr > 0) || (u < orc_exp(lr));
            } else if (alg == ORC_GLAUBER) {
                flip = u < orc_logistic(-beta * dE);
            } else {
                int up = u < orc_logistic((beta * (double)so) * dE);
                flip = up != (so == 1);
            }
            if (flip) sn = -so;
        } else if (alg == ORC_HEATBATH) {
            double c = bcg_coupling(s, v, rowptr, col, Jv, J);
            double hf = (hv || h != 0.0) ? bcg_field(v, hv, h) : 0.0;
            double e1 = (c - hf * (-1.0)) + D;
            double e3 = (-c - hf) + D;
            double w1 = orc_exp(-beta * e1), w2 = orc_exp(-beta * 0.0), w3 = orc_exp(-beta * e3);
            double z = (w1 + w2) + w3;
            double r = u * z;
            sn = r < w1 ? -1 : (r < w1 + w2 ? 0 : 1);
            if (sn != so) dE = orc_bcg_delta_energy(s, v, sn, rowptr, col, Jv, J, D, hv, h);
        } else {
            uint32_t c2[4] = {(uint32_t)a, (uint32_t)(a >> 32), (uint32_t)P_SEQ2 << 24, stream}, w2[4];
            orc_philox4x32_10(c2, key, w2);
            int prop = bc_propose(so, (int)(w2[0] >> 31));
            dE = orc_bcg_delta_energy(s, v, prop, rowptr, col, Jv, J, D, hv, h);
            double lr = -beta * dE;
            int acc = alg == ORC_METROPOLIS ? ((lr > 0) || (u < orc_exp(lr))) : (u < orc_logistic(lr));
            if (acc) sn = prop;
        }
        if (sn != so) {
            s[v] = (int8_t)sn;
            *E += dE;
            *M += sn - so;
            ++acc_n;
        }
    }
    *attempts += (uint64_t)nattempts;
    *accepts += acc_n;
    return ORC_OK;
}

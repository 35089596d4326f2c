/*
 * mcx_oracle.h -- CPU oracle for the spin-flip hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, includes or
 * calls this code; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it, as the checker.  It is a plain-C restatement of the
 * MonteCarloX.jl / SpinSystems algorithms for this path (citations beside each
 * function in mcx_oracle.c), written independently of the CUDA kernels.
 *
 * Two modes:
 *   (i)  checkerboard order fed by a Philox4x32-10 stream per (site, sweep,
 *        colour, purpose); uint32 threshold tables for the canonical rules.
 *        This is the bit-exact target for the device.
 *   (ii) the reference's own sequential random-site order (pick_site + FP64
 *        exp / logistic decisions), for statistics and for the CPU baseline.
 */
#ifndef MCX_ORACLE_H
#define MCX_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_OK = 0, ORC_ERR_INVALID = 1, ORC_ERR_RANGE = 2 };
enum { ORC_ISING = 0, ORC_BC = 1 };
enum { ORC_METROPOLIS = 0, ORC_GLAUBER = 1, ORC_HEATBATH = 2 };
enum { ORC_MUCA = 0, ORC_WL = 1 };

/* Philox4x32-10, Salmon, Moraes, Dror, Shaw, SC'11. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* the per-site word used by the checkerboard mode */
uint32_t orc_site_word(uint64_t seed, uint32_t stream, uint64_t sweep, int colour,
                       int purpose, uint64_t site);
/* natural logarithm restated from the atanh series; used for every FP64 decision */
double orc_log(double x);
void orc_log_array(const double* x, double* y, int64_t n);

/* acceptance tables (uint32 thresholds widened to u64 so 2^32 means "always") */
int orc_table_ising(int dim, int alg, double beta, double J, double h,
                    uint64_t* thr /*2*(2d+1)*/, uint32_t* xmask /*2*(2d+1)*/);
int orc_table_bc(int dim, int alg, double beta, double J, double D, double h,
                 uint64_t* thr /*metropolis/glauber: 3*2*(4d+1); heatbath: 2*(4d+1)*/);

void orc_init_random(int8_t* s, int model, int dim, const int32_t* L, uint64_t seed,
                     uint32_t stream);
void orc_observables(const int8_t* s, int dim, const int32_t* L, int64_t* P, int64_t* M,
                     int64_t* Q);

int orc_cb_sweep(int8_t* s, int model, int dim, const int32_t* L, int alg, double beta,
                 double J, double D, double h, uint64_t seed, uint32_t stream,
                 uint64_t sweep0, int64_t nsweeps, int64_t* obs /* nsweeps*3 or NULL */,
                 uint64_t* attempts, uint64_t* accepts);

/* orc_cb_sweep with the uniforms form (0 per-site words, 1 bit planes) */
int orc_cb_sweep_u(int8_t* s, int model, int dim, const int32_t* L, int alg, double beta,
                   double J, double D, double h, uint64_t seed, uint32_t stream,
                   uint64_t sweep0, int64_t nsweeps, int64_t* obs, uint64_t* attempts,
                   uint64_t* accepts, int uniforms);
/* the Blume-Capel proposal bit of colour-class site e under bit-plane uniforms */
int orc_bc_plane_bit(uint64_t seed, uint32_t stream, uint64_t sweep, int colour, uint64_t e);
/* the bit-plane uniform of colour-class site e (e = linear index >> 1) */
uint32_t orc_plane_uniform(uint64_t seed, uint32_t stream, uint64_t sweep, int colour, uint64_t e);

int orc_seq_attempts(int8_t* s, int model, int dim, const int32_t* L, int alg, double beta,
                     double J, double D, double h, uint64_t seed, uint32_t stream,
                     uint64_t attempt0, int64_t nattempts, uint64_t* steps,
                     uint64_t* accepted);

int orc_flathist_sweep(int8_t* s, int model, int dim, const int32_t* L, double J, double D,
                       double h, int mode, double* lnw, int64_t* H, int64_t start,
                       int64_t step, int64_t nbins, double logf, uint64_t seed,
                       uint32_t stream, uint64_t sweep0, int64_t nsweeps, int64_t* obs,
                       uint64_t* steps, uint64_t* accepted);
int orc_flathist_trace(int8_t* s, int model, int dim, const int32_t* L, double J, double D,
                       double h, int mode, double* lnw, int64_t* H, int64_t start,
                       int64_t step, int64_t nbins, double logf, uint64_t seed,
                       uint32_t stream, uint64_t sweep0, int64_t nsweeps, double* tr_u,
                       double* tr_lr, int64_t tr_cap, int64_t* tr_n);
void orc_muca_update(double* lnw, const int64_t* H, int64_t nbins);
int orc_wl_flat(const int64_t* H, const uint8_t* visited, int64_t nbins, double flatness,
                double* ratio);

int orc_pt_exchange(int n, const double* betas, int32_t* pos, int32_t* stage,
                    const double* x, uint64_t seed, uint32_t ladder, uint64_t t,
                    uint64_t* steps, uint64_t* accepted);

/* general graphs and couplings (IsingGraph / IsingMatrix); Jv / hv may be NULL */
double orc_exp(double x);
double orc_logistic(double x);
int orc_graph_colour(int64_t n, const int64_t* rowptr, const int32_t* col, int32_t* colour);
void orc_graph_init_random(int8_t* s, int64_t n, uint64_t seed, uint32_t stream);
double orc_graph_delta_energy(const int8_t* s, int64_t v, const int64_t* rowptr,
                              const int32_t* col, const double* Jv, double J, const double* hv,
                              double h);
void orc_graph_observables(const int8_t* s, int64_t n, const int64_t* rowptr, const int32_t* col,
                           const double* Jv, double J, const double* hv, double h, double* E,
                           int64_t* M);
int orc_graph_sweep(int8_t* s, int64_t n, const int64_t* rowptr, const int32_t* col,
                    const double* Jv, double J, const double* hv, double h, int alg, double beta,
                    uint64_t seed, uint32_t stream, uint64_t sweep0, int64_t nsweeps, double* E,
                    int64_t* M, double* E_series, int64_t* M_series, uint64_t* attempts,
                    uint64_t* accepts);

/* Blume-Capel on general graphs (BlumeCapelGraph / BlumeCapelMatrix); Jv / hv may be NULL */
double orc_bcg_delta_energy(const int8_t* s, int64_t v, int s_new, const int64_t* rowptr,
                            const int32_t* col, const double* Jv, double J, double D,
                            const double* hv, double h);
void orc_bcg_observables(const int8_t* s, int64_t n, const int64_t* rowptr, const int32_t* col,
                         const double* Jv, double J, double D, const double* hv, double h,
                         double* E, int64_t* M);
void orc_bcg_init_random(int8_t* s, int64_t n, uint64_t seed, uint32_t stream);
int orc_bcg_sweep(int8_t* s, int64_t n, const int64_t* rowptr, const int32_t* col,
                  const double* Jv, double J, double D, const double* hv, double h, int alg,
                  double beta, uint64_t seed, uint32_t stream, uint64_t sweep0, int64_t nsweeps,
                  double* E, int64_t* M, double* E_series, int64_t* M_series, uint64_t* attempts,
                  uint64_t* accepts);
int orc_graph_seq_attempts(int8_t* s, int64_t n, const int64_t* rowptr, const int32_t* col,
                           const double* Jv, double J, const double* hv, double h, int bc, double D,
                           int alg, double beta, uint64_t seed, uint32_t stream, uint64_t attempt0,
                           int64_t nattempts, double* E, int64_t* M, uint64_t* attempts,
                           uint64_t* accepts);

/* integrated autocorrelation time (-1 on invalid arguments) */
double orc_tau_int(const double* x, int64_t n, int64_t max_lag, double c);

/* CPU baseline: nthreads independent chains in sequential random-site order */
int orc_bench_seq(int model, int dim, const int32_t* L, int alg, double beta, double J,
                  double D, double h, uint64_t seed, int nthreads, int64_t attempts_per_thread,
                  double* seconds);

#ifdef __cplusplus
}
#endif
#endif

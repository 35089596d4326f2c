// mcx_internal.h -- host-side internals shared by the libmcx_cuda translation units.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/mcx.h"

namespace mcx {

// Philox counter word 2 carries (sweep hi16 | colour<<16 | purpose<<24).
enum Purpose : uint32_t {
    P_ACCEPT = 0,   // acceptance / heat-bath word of a site
    P_PROPOSE = 1,  // Blume-Capel proposal bit (top bit of the word)
    P_LOW = 2,      // low word of a 53-bit uniform (flat-histogram decisions)
    P_INIT = 3,     // init!(sys, :random)
    P_EXCHANGE = 4,  // replica-exchange uniform
    P_GRAPH = 7,     // 53-bit uniform of a site of a general graph (words 0 and 1)
    P_GRAPH_INIT = 8,  // init!(sys, :random) of a general graph
    P_PLANES = 9,      // bit planes 0..7 of the MCX_UNIFORMS_PLANES uniforms (four blocks per 64 sites)
    P_TAIL = 10        // low 24 bits of a MCX_UNIFORMS_PLANES uniform (word e & 3 of block e >> 2)
};

void set_error(const char* fmt, ...);
mcx_status fail(mcx_status st, const char* fmt, ...);
mcx_status cuda_fail(cudaError_t e, const char* what);

#define MCX_CUDA(call)                                             \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return ::mcx::cuda_fail(_e, #call); \
    } while (0)

#define MCX_CHECK(expr)                       \
    do {                                      \
        mcx_status _s = (expr);               \
        if (_s != MCX_OK) return _s;          \
    } while (0)

// Largest acceptance table: Blume-Capel Metropolis in 3-D has 3*2*13 entries.
constexpr int kMaxTable = 80;

struct Table {
    uint64_t thr[kMaxTable];  // 2^32 means "always"
    int n;
};

// Host-side table construction (same rules as the reference; see mcx_tables.cu).
mcx_status build_ising_table(int dim, mcx_algorithm alg, double beta, double J, double h,
                             Table* t);
mcx_status build_bc_table(int dim, mcx_algorithm alg, double beta, double J, double D,
                          double h, Table* t);

}  // namespace mcx

struct mcx_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint64_t budget = 0;
    uint64_t used = 0;
    uint64_t launches = 0;
    int num_sms = 0;
    cudaStream_t capture_stream = nullptr;  // private stream for CUDA-graph capture
    void* d_scratch = nullptr;              // per-call descriptors (walkers), grown on demand
    size_t scratch_bytes = 0;
    // the caller's handle plus one per live object created on this context: the
    // streams and the accounting stay valid until the last of them is destroyed, in
    // whatever order a garbage collector finalises them
    std::atomic<int> refs{1};
};

namespace mcx {
void ctx_release(mcx_ctx* ctx);
// Device scratch of at least `bytes` owned by the context (valid until the next call on
// the same context; contexts are used by one thread at a time).
mcx_status ctx_scratch(mcx_ctx* ctx, size_t bytes, void** out);

// Reference to the context held by every object created on it.
struct CtxHold {
    mcx_ctx* p = nullptr;
    CtxHold() = default;
    CtxHold(const CtxHold&) = delete;
    CtxHold& operator=(const CtxHold&) = delete;
    void set(mcx_ctx* c) {
        if (c) c->refs.fetch_add(1);
        if (p) ctx_release(p);
        p = c;
    }
    ~CtxHold() {
        if (p) ctx_release(p);
    }
};
}  // namespace mcx

struct mcx_lattice {
    mcx_ctx* ctx = nullptr;
    mcx::CtxHold hold;  // keeps ctx alive while the lattice exists
    mcx_model model = MCX_ISING;
    mcx_layout layout = MCX_LAYOUT_INT8;
    int dim = 2;
    int64_t L[3] = {1, 1, 1};
    double J = 1, D = 0, h = 0;
    int64_t N = 0;       // sites
    int64_t W = 0;       // sites of one colour per row (Lx/2)
    int64_t rows = 0;    // Ly*Lz
    // INT8 layout: colour-split arrays, row r = y + Ly*z, entry k <-> x = 2k + ((y+z+c)&1)
    int8_t* d_col[2] = {nullptr, nullptr};
    // MSC64 layout: same order, bit b of word w <-> k = 64*w + b
    unsigned long long* d_msc[2] = {nullptr, nullptr};
    int8_t* d_lin = nullptr;       // staging buffer in linear order (set/get)
    int64_t* d_state = nullptr;    // current (pair_sum, spin_sum, spin2_sum)
    unsigned long long* d_acc = nullptr;  // accepted-move counter
    int64_t* d_series = nullptr;   // per-sweep deltas, then the running series
    int64_t series_cap = 0;        // in sweeps
    int64_t series_len = 0;        // sweeps recorded by the last mcx_sweep
    int64_t device_bytes = 0;
    int tuned_V = 0;               // row width chosen by mcx_autotune (0 = default)
    int allow_packing = 1;         // int8: multi-sweep calls may use a transient MSC64 copy
    int uniforms = 0;              // mcx_uniforms of rank-form Metropolis sweeps
    int cluster_size = 0;          // CTAs of the last cluster-form call (0: not tried, -1: none fits)
    // that call's kernel, block size and shared memory, reused while its key (heat bath,
    // 32-bit table) is the same, so later calls skip the occupancy query (about 1 us of the
    // ~32 us a one-sweep call through the Python mirror costs on a GB300 host)
    int cluster_key = -1;
    const void* cluster_fn = nullptr;
    int cluster_threads = 0;
    size_t cluster_smem = 0;
    unsigned long long* d_sweep_base = nullptr;  // {first sweep, seed, stream, series offset} read by captured graphs
    struct Graph {
        int alg;
        int uniforms;  // the captured arguments carry the form (Blume-Capel proposals)
        double beta;
        int64_t nsweeps;
        int V;
        const int64_t* series;
        cudaGraphExec_t exec;
    };
    std::vector<Graph> graphs;     // instantiated sweep sequences (most recent last)
};

namespace mcx {
// A per-sweep series read in place by the autocorrelation kernel: sample t is
// base[t * stride] (float64) or sum_k coef[k] * base[t * stride + k] (int64 columns).
enum TraceType { TRACE_F64 = 0, TRACE_I64 = 1 };
struct TraceSrc {
    const void* base;       // device address of sample 0; nullptr: host values at host_offset
    long long n, stride;
    long long cap;          // lag window
    long long host_offset;
    int type, ncols, skip, pad;
    double coef[3];
};
// integrated autocorrelation times of the traces (NaN for skipped ones); waits.
mcx_status launch_tau_int(mcx_ctx* ctx, const std::vector<TraceSrc>& srcs, const double* host_values,
                          size_t host_count, double c, double* taus);
// the batch lag-window rules: cap = min(max_lag, n/2) (max_lag <= 0: n/2); skip when
// n < min_points or cap < 1
void tau_window(TraceSrc& s, long long n, long long min_points, long long max_lag);

mcx_status dev_alloc(mcx_ctx* ctx, void** p, size_t bytes);
void dev_free(mcx_ctx* ctx, void* p, size_t bytes);
// launch accounting helper
inline void count_launch(mcx_ctx* ctx, uint64_t n = 1) { ctx->launches += n; }
mcx_status ensure_series(mcx_lattice* lat, int64_t nsweeps);
mcx_status recompute_state(mcx_lattice* lat);
// enqueue kernels that finish a run: prefix-sum the per-sweep deltas into the series
mcx_status finish_series(mcx_lattice* lat, int64_t nsweeps);
mcx_status launch_prefix(mcx_lattice* lat, int64_t nsweeps, cudaStream_t stream);
void clear_graphs(mcx_lattice* lat);
}  // namespace mcx

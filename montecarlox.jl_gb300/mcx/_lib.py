"""ctypes binding of libmcx_cuda (the C ABI declared in include/mcx.h).

The library is built in-tree by ``montecarlox.jl_gb300/build.py``.  There is no
CPU fallback: if the shared library is missing, importing any compute entry point
raises.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libmcx_cuda.so")

MCX_OK = 0
MCX_ERR_INVALID_ARG = 1
MCX_ERR_OUT_OF_RANGE = 2
MCX_ERR_OOM = 3
MCX_ERR_BUDGET = 4
MCX_ERR_TIMEOUT = 5
MCX_ERR_CUDA = 6
MCX_ERR_NOT_READY = 7
MCX_ERR_NOT_FOUND = 8

ISING, BLUME_CAPEL = 0, 1
METROPOLIS, GLAUBER, HEATBATH = 0, 1, 2
LAYOUT_INT8, LAYOUT_MSC64 = 0, 1
MUCA, WANG_LANDAU = 0, 1


class mcx_config(C.Structure):
    _fields_ = [("device", C.c_int), ("stream", C.c_void_p), ("hbm_budget", C.c_uint64)]


class mcx_rng(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("counter", C.c_uint64), ("stream", C.c_uint32),
                ("reserved", C.c_uint32)]


class mcx_counters(C.Structure):
    _fields_ = [("attempts", C.c_uint64), ("accepted", C.c_uint64)]


_P = C.c_void_p
_i64p = C.POINTER(C.c_int64)
_u64p = C.POINTER(C.c_uint64)
_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)

# name -> (restype, argtypes)
SIGNATURES = {
    "mcx_status_string": (C.c_char_p, [C.c_int]),
    "mcx_last_error_string": (C.c_char_p, []),
    "mcx_version": (C.c_int, []),
    "mcx_ctx_create": (C.c_int, [C.POINTER(mcx_config), C.POINTER(_P)]),
    "mcx_ctx_destroy": (C.c_int, [_P]),
    "mcx_sync": (C.c_int, [_P]),
    "mcx_ctx_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "mcx_ctx_memory": (C.c_int, [_P, _u64p, _u64p]),
    "mcx_ctx_launches": (C.c_int, [_P, _u64p]),
    "mcx_lattice_create": (C.c_int, [_P, C.c_int, C.c_int, _i32p, C.c_int, C.c_double, C.c_double,
                                     C.c_double, C.POINTER(_P)]),
    "mcx_lattice_destroy": (C.c_int, [_P]),
    "mcx_lattice_info": (C.c_int, [_P, _i64p, _i64p]),
    "mcx_set_spins": (C.c_int, [_P, _P, C.c_size_t]),
    "mcx_get_spins": (C.c_int, [_P, _P, C.c_size_t]),
    "mcx_init_random": (C.c_int, [_P, C.c_uint64, C.c_uint32]),
    "mcx_init_uniform": (C.c_int, [_P, C.c_int8]),
    "mcx_observables": (C.c_int, [_P, _i64p, _i64p, _i64p]),
    "mcx_recompute_observables": (C.c_int, [_P, _i64p, _i64p, _i64p]),
    "mcx_energy": (C.c_int, [_P, _f64p, _i64p]),
    "mcx_sweep": (C.c_int, [_P, C.c_int, C.c_double, C.POINTER(mcx_rng), C.c_int64, _P,
                            C.POINTER(mcx_counters)]),
    "mcx_read_series": (C.c_int, [_P, _P, C.c_int64]),
    "mcx_spin_flip": (C.c_int, [_P, C.c_int, C.c_double, C.POINTER(mcx_rng), C.c_int64, C.POINTER(mcx_counters)]),
    "mcx_graph_spin_flip": (C.c_int, [_P, C.c_int, C.c_double, C.POINTER(mcx_rng), C.c_int64,
                                      C.POINTER(mcx_counters)]),
    "mcx_sweep_batch": (C.c_int, [C.POINTER(_P), C.c_int32, C.c_int, _f64p, C.POINTER(mcx_rng), C.c_int64,
                                  C.POINTER(C.c_void_p), C.POINTER(mcx_counters)]),
    "mcx_autotune": (C.c_int, [_P, C.c_int, C.c_double, _i32p, _f64p]),
    "mcx_lattice_set_packing": (C.c_int, [_P, C.c_int32]),
    "mcx_lattice_set_uniforms": (C.c_int, [_P, C.c_int32]),
    "mcx_flathist_create": (C.c_int, [_P, C.c_int64, C.c_int64, C.c_int64, C.POINTER(_P)]),
    "mcx_flathist_destroy": (C.c_int, [_P]),
    "mcx_flathist_set_logweight": (C.c_int, [_P, _P, C.c_int64]),
    "mcx_flathist_get_logweight": (C.c_int, [_P, _P, C.c_int64]),
    "mcx_flathist_set_histogram": (C.c_int, [_P, _P, C.c_int64]),
    "mcx_flathist_get_histogram": (C.c_int, [_P, _P, C.c_int64]),
    "mcx_flathist_reset": (C.c_int, [_P]),
    "mcx_flathist_reweight": (C.c_int, [_P, _P, C.c_int32, _P, _P, _P, _P, C.c_int64]),
    "mcx_flathist_update_muca": (C.c_int, [_P]),
    "mcx_flathist_flatness": (C.c_int, [_P, C.c_double, C.POINTER(C.c_int), _f64p]),
    "mcx_flathist_merge": (C.c_int, [_P, C.POINTER(_P), C.c_int]),
    "mcx_flathist_copy_logweight": (C.c_int, [_P, _P]),
    "mcx_flathist_sweep": (C.c_int, [C.POINTER(_P), C.c_int, C.POINTER(_P), C.c_int, C.c_int, C.c_double,
                                     C.POINTER(mcx_rng), C.c_int64, C.POINTER(mcx_counters)]),
    "mcx_server_create": (C.c_int, [_P, C.c_uint64, C.c_int32, C.c_int32, C.POINTER(_P)]),
    "mcx_server_destroy": (C.c_int, [_P]),
    "mcx_server_submit": (C.c_int, [_P, _P, _u64p]),
    "mcx_server_step": (C.c_int, [_P, _i32p, _i32p]),
    "mcx_server_poll": (C.c_int, [_P, C.c_uint64, _P]),
    "mcx_server_cancel": (C.c_int, [_P, C.c_uint64]),
    "mcx_server_start": (C.c_int, [_P]),
    "mcx_server_stop": (C.c_int, [_P, C.c_double]),
    "mcx_server_set_loop_limits": (C.c_int, [_P, C.c_int64, C.c_int64]),
    "mcx_server_loop_info": (C.c_int, [_P, _i32p, _i32p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64),
                                       C.POINTER(C.c_uint64)]),
    "mcx_poll_flag": (C.c_int, [_P, C.c_uint32, C.c_int64, C.c_int64]),
    "mcx_server_get_stats": (C.c_int, [_P, _P]),
    "mcx_sweep_noalloc": (C.c_int, [_P, C.c_int, C.c_double, C.POINTER(mcx_rng), C.c_int64, _P, _P]),
    "mcx_pt_create": (C.c_int, [_P, C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_double, C.c_double,
                                C.POINTER(_P)]),
    "mcx_pt_destroy": (C.c_int, [_P]),
    "mcx_pt_info": (C.c_int, [_P, _i32p, _i64p, _i64p]),
    "mcx_pt_init_random": (C.c_int, [_P, C.c_uint64]),
    "mcx_pt_set_spins": (C.c_int, [_P, C.c_int32, _P, C.c_size_t]),
    "mcx_pt_get_spins": (C.c_int, [_P, C.c_int32, _P, C.c_size_t]),
    "mcx_pt_run": (C.c_int, [_P, C.c_int, C.POINTER(mcx_rng), C.c_int64, C.c_int32, C.c_int, _P]),
    "mcx_pt_indices": (C.c_int, [_P, _P, _i32p]),
    "mcx_pt_exchange_counters": (C.c_int, [_P, _P, _P]),
    "mcx_pt_observables": (C.c_int, [_P, _P, _P]),
    "mcx_pt_replica_accepted": (C.c_int, [_P, _P]),
    "mcx_pt_set_schedule": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "mcx_pt_get_schedule": (C.c_int, [_P, _i32p, _i32p, _i32p, _i32p]),
    "mcx_pt_autotune": (C.c_int, [_P, C.c_int, C.c_int32, C.c_int32, _i32p, _i32p, _i32p, _f64p]),
    "mcx_pt_set_wait_limit": (C.c_int, [_P, C.c_int64]),
    "mcx_pt_set_indices": (C.c_int, [_P, _P, C.c_int32]),
    "mcx_pt_set_exchange_counters": (C.c_int, [_P, _P, _P]),
    "mcx_flathist_get_visited": (C.c_int, [_P, _P, C.c_int64]),
    "mcx_flathist_set_visited": (C.c_int, [_P, _P, C.c_int64]),
    "mcx_wait_flag_test": (C.c_int, [_P, C.c_int64]),
    "mcx_graph_create": (C.c_int, [_P, C.c_int64, _P, _P, _P, C.c_double, _P, C.c_double, C.POINTER(_P)]),
    "mcx_graph_destroy": (C.c_int, [_P]),
    "mcx_bcgraph_create": (C.c_int, [_P, C.c_int64, _P, _P, _P, C.c_double, C.c_double, _P, C.c_double,
                                     C.POINTER(_P)]),
    "mcx_graph_delta_energy_to": (C.c_int, [_P, C.c_int64, C.c_int8, _f64p]),
    "mcx_graph_set_site": (C.c_int, [_P, C.c_int64, C.c_int8]),
    "mcx_graph_info": (C.c_int, [_P, _i64p, _i32p, _i64p, _i64p]),
    "mcx_graph_colours": (C.c_int, [_P, _P, C.c_size_t]),
    "mcx_graph_set_spins": (C.c_int, [_P, _P, C.c_size_t]),
    "mcx_graph_get_spins": (C.c_int, [_P, _P, C.c_size_t]),
    "mcx_graph_init_random": (C.c_int, [_P, C.c_uint64, C.c_uint32]),
    "mcx_graph_init_uniform": (C.c_int, [_P, C.c_int8]),
    "mcx_graph_energy": (C.c_int, [_P, C.c_int, _f64p, _i64p]),
    "mcx_graph_delta_energy": (C.c_int, [_P, C.c_int64, _f64p]),
    "mcx_graph_flip": (C.c_int, [_P, C.c_int64]),
    "mcx_graph_sweep": (C.c_int, [_P, C.c_int, C.c_double, C.POINTER(mcx_rng), C.c_int64, _P, _P,
                                  C.POINTER(mcx_counters)]),
    "mcx_tau_int": (C.c_int, [_P, _P, _P, C.c_int32, C.c_int64, C.c_int64, C.c_double, _P]),
    "mcx_lattice_tau_int": (C.c_int, [_P, C.c_int, C.c_int64, C.c_double, _f64p]),
    "mcx_graph_tau_int": (C.c_int, [_P, C.c_int, C.c_int64, C.c_double, _f64p]),
    "mcx_pt_set_record": (C.c_int, [_P, C.c_int32]),
    "mcx_pt_tau_int": (C.c_int, [_P, C.c_int, C.c_int64, C.c_int64, C.c_double, _P]),
    "mcx_ladder_exchange": (C.c_int, [C.c_int32, _P, _P, _P, C.c_double, C.c_double, _P, _i32p, C.c_uint64,
                                      C.c_int32, C.c_uint64, _P, _P]),
}

PT_PERSISTENT, PT_PLAIN = 0, 1
JOB_CANONICAL, JOB_MULTICANONICAL = 0, 1


class mcx_job(C.Structure):
    _fields_ = [("model", C.c_int32), ("dim", C.c_int32), ("L", C.c_int32 * 3), ("kind", C.c_int32),
                ("alg", C.c_int32), ("reserved0", C.c_int32), ("beta", C.c_double), ("J", C.c_double),
                ("D", C.c_double), ("h", C.c_double), ("seed", C.c_uint64), ("stream", C.c_uint32),
                ("reserved1", C.c_uint32), ("nsweeps", C.c_int64), ("bin_start", C.c_int64),
                ("bin_step", C.c_int64), ("nbins", C.c_int64), ("logweight", C.c_void_p),
                ("obs_series", C.c_void_p), ("histogram", C.c_void_p), ("logweight_out", C.c_void_p),
                ("final_spins", C.c_void_p)]


class mcx_job_result(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("pair_sum", C.c_int64), ("spin_sum", C.c_int64),
                ("spin2_sum", C.c_int64), ("attempts", C.c_uint64), ("accepted", C.c_uint64),
                ("sweeps_done", C.c_int64), ("submit_s", C.c_double), ("admit_s", C.c_double),
                ("finish_s", C.c_double)]


class mcx_server_stats(C.Structure):
    _fields_ = [("active", C.c_int32), ("pending", C.c_int32), ("iterations", C.c_uint64),
                ("jobs_done", C.c_uint64), ("attempts_done", C.c_uint64), ("bytes_in_use", C.c_uint64),
                ("peak_bytes", C.c_uint64), ("now_s", C.c_double)]

_lib = None


def load(path: str = LIB_PATH):
    """Load libmcx_cuda.so; raises OSError (no fallback) when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError("libmcx_cuda.so not found at %s: build it with montecarlox.jl_gb300/build.py "
                      "(there is no CPU fallback)" % path)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def error_string() -> str:
    return load().mcx_last_error_string().decode(errors="replace")

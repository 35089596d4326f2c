"""CPU oracle for the spin-flip hot path -- TEST INFRASTRUCTURE ONLY.

The C restatement in ``mcx_oracle.c`` is the checker for the CUDA library.  Only
``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
may import this package.  The product library never calls it.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

ISING, BC = 0, 1
METROPOLIS, GLAUBER, HEATBATH = 0, 1, 2
MUCA, WL = 0, 1
OK, ERR_INVALID, ERR_RANGE = 0, 1, 2

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        u32p = np.ctypeslib.ndpointer(np.uint32, flags="C")
        u64p = np.ctypeslib.ndpointer(np.uint64, flags="C")
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
        i8p = np.ctypeslib.ndpointer(np.int8, flags="C")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
        u8p = np.ctypeslib.ndpointer(np.uint8, flags="C")
        L.orc_philox4x32_10.argtypes = [u32p, u32p, u32p]
        L.orc_site_word.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_int, C.c_int, C.c_uint64]
        L.orc_site_word.restype = C.c_uint32
        L.orc_log.argtypes = [C.c_double]
        L.orc_log.restype = C.c_double
        L.orc_log_array.argtypes = [f64p, f64p, C.c_int64]
        L.orc_log_array.restype = None
        L.orc_table_ising.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, u64p, u32p]
        L.orc_table_bc.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, u64p]
        L.orc_init_random.argtypes = [i8p, C.c_int, C.c_int, i32p, C.c_uint64, C.c_uint32]
        L.orc_init_random.restype = None
        L.orc_observables.argtypes = [i8p, C.c_int, i32p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64)]
        L.orc_observables.restype = None
        L.orc_cb_sweep.argtypes = [i8p, C.c_int, C.c_int, i32p, C.c_int, C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_uint64, C.c_uint32, C.c_uint64, C.c_int64, C.c_void_p,
                                   C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.orc_cb_sweep_u.argtypes = L.orc_cb_sweep.argtypes + [C.c_int]
        L.orc_plane_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_int, C.c_uint64]
        L.orc_plane_uniform.restype = C.c_uint32
        L.orc_bc_plane_bit.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_int, C.c_uint64]
        L.orc_bc_plane_bit.restype = C.c_int
        L.orc_seq_attempts.argtypes = [i8p, C.c_int, C.c_int, i32p, C.c_int, C.c_double, C.c_double,
                                       C.c_double, C.c_double, C.c_uint64, C.c_uint32, C.c_uint64, C.c_int64,
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.orc_flathist_sweep.argtypes = [i8p, C.c_int, C.c_int, i32p, C.c_double, C.c_double, C.c_double,
                                         C.c_int, f64p, i64p, C.c_int64, C.c_int64, C.c_int64, C.c_double,
                                         C.c_uint64, C.c_uint32, C.c_uint64, C.c_int64, C.c_void_p,
                                         C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.orc_flathist_trace.argtypes = [i8p, C.c_int, C.c_int, i32p, C.c_double, C.c_double, C.c_double,
                                         C.c_int, f64p, i64p, C.c_int64, C.c_int64, C.c_int64, C.c_double,
                                         C.c_uint64, C.c_uint32, C.c_uint64, C.c_int64, f64p, f64p, C.c_int64,
                                         C.POINTER(C.c_int64)]
        L.orc_muca_update.argtypes = [f64p, i64p, C.c_int64]
        L.orc_muca_update.restype = None
        L.orc_wl_flat.argtypes = [i64p, u8p, C.c_int64, C.c_double, C.POINTER(C.c_double)]
        L.orc_pt_exchange.argtypes = [C.c_int, f64p, i32p, C.POINTER(C.c_int32), f64p, C.c_uint64,
                                      C.c_uint32, C.c_uint64, u64p, u64p]
        L.orc_bench_seq.argtypes = [C.c_int, C.c_int, i32p, C.c_int, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_uint64, C.c_int, C.c_int64, C.POINTER(C.c_double)]
        vp = C.c_void_p
        L.orc_exp.argtypes = [C.c_double]
        L.orc_exp.restype = C.c_double
        L.orc_logistic.argtypes = [C.c_double]
        L.orc_logistic.restype = C.c_double
        L.orc_graph_colour.argtypes = [C.c_int64, i64p, i32p, i32p]
        L.orc_graph_init_random.argtypes = [i8p, C.c_int64, C.c_uint64, C.c_uint32]
        L.orc_graph_init_random.restype = None
        L.orc_graph_delta_energy.argtypes = [i8p, C.c_int64, i64p, i32p, vp, C.c_double, vp, C.c_double]
        L.orc_graph_delta_energy.restype = C.c_double
        L.orc_graph_observables.argtypes = [i8p, C.c_int64, i64p, i32p, vp, C.c_double, vp, C.c_double,
                                            C.POINTER(C.c_double), C.POINTER(C.c_int64)]
        L.orc_graph_observables.restype = None
        L.orc_graph_sweep.argtypes = [i8p, C.c_int64, i64p, i32p, vp, C.c_double, vp, C.c_double, C.c_int,
                                      C.c_double, C.c_uint64, C.c_uint32, C.c_uint64, C.c_int64,
                                      C.POINTER(C.c_double), C.POINTER(C.c_int64), vp, vp,
                                      C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.orc_bcg_delta_energy.argtypes = [i8p, C.c_int64, C.c_int, i64p, i32p, vp, C.c_double, C.c_double, vp,
                                           C.c_double]
        L.orc_bcg_delta_energy.restype = C.c_double
        L.orc_bcg_observables.argtypes = [i8p, C.c_int64, i64p, i32p, vp, C.c_double, C.c_double, vp, C.c_double,
                                          C.POINTER(C.c_double), C.POINTER(C.c_int64)]
        L.orc_bcg_observables.restype = None
        L.orc_bcg_init_random.argtypes = [i8p, C.c_int64, C.c_uint64, C.c_uint32]
        L.orc_bcg_init_random.restype = None
        L.orc_bcg_sweep.argtypes = [i8p, C.c_int64, i64p, i32p, vp, C.c_double, C.c_double, vp, C.c_double, C.c_int,
                                    C.c_double, C.c_uint64, C.c_uint32, C.c_uint64, C.c_int64,
                                    C.POINTER(C.c_double), C.POINTER(C.c_int64), vp, vp, C.POINTER(C.c_uint64),
                                    C.POINTER(C.c_uint64)]
        L.orc_graph_seq_attempts.argtypes = [i8p, C.c_int64, i64p, i32p, vp, C.c_double, vp, C.c_double, C.c_int,
                                             C.c_double, C.c_int, C.c_double, C.c_uint64, C.c_uint32, C.c_uint64,
                                             C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                             C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.orc_tau_int.argtypes = [f64p, C.c_int64, C.c_int64, C.c_double]
        L.orc_tau_int.restype = C.c_double
        _lib = L
    return _lib


def _dims(L):
    L = [int(v) for v in L]
    return len(L), np.array(L + [1] * (3 - len(L)), dtype=np.int32)


def philox(ctr, key):
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out


def site_word(seed, stream, sweep, colour, purpose, site):
    return int(lib().orc_site_word(seed, stream, sweep, colour, purpose, site))


def log(x):
    return float(lib().orc_log(float(x)))


def log_array(x):
    """The project log (the one the device uses) of every element."""
    x = np.ascontiguousarray(x, np.float64)
    y = np.empty_like(x)
    lib().orc_log_array(x, y, x.size)
    return y


def table_ising(dim, alg, beta, J=1.0, h=0.0):
    n = 2 * (2 * dim + 1)
    thr = np.zeros(n, np.uint64)
    xm = np.zeros(n, np.uint32)
    rc = lib().orc_table_ising(dim, alg, beta, J, h, thr, xm)
    assert rc == OK
    return thr, xm


def table_bc(dim, alg, beta, J=1.0, D=1.0, h=0.0):
    n = 3 * 2 * (4 * dim + 1)
    thr = np.zeros(n, np.uint64)
    rc = lib().orc_table_bc(dim, alg, beta, J, D, h, thr)
    assert rc == OK
    return thr


def init_random(model, L, seed, stream=0):
    dim, Lv = _dims(L)
    s = np.zeros(int(np.prod(L)), np.int8)
    lib().orc_init_random(s, model, dim, Lv, seed, stream)
    return s


def observables(s, L):
    dim, Lv = _dims(L)
    P, M, Q = C.c_int64(), C.c_int64(), C.c_int64()
    lib().orc_observables(np.ascontiguousarray(s, np.int8), dim, Lv, C.byref(P), C.byref(M), C.byref(Q))
    return P.value, M.value, Q.value


def cb_sweep(s, model, L, alg, beta, seed, stream=0, sweep0=0, nsweeps=1, J=1.0, D=0.0, h=0.0,
             record=True, uniforms=0):
    """Checkerboard sweeps in place on ``s``; returns (obs[nsweeps,3] or None, attempts, accepts).
    ``uniforms``: 0 per-site Philox words, 1 bit-plane uniforms for the rank-form rules."""
    dim, Lv = _dims(L)
    obs = np.zeros((nsweeps, 3), np.int64) if record else None
    att, acc = C.c_uint64(0), C.c_uint64(0)
    args = (s, model, dim, Lv, alg, beta, J, D, h, seed, stream, sweep0, nsweeps,
            obs.ctypes.data if record else None, C.byref(att), C.byref(acc))
    rc = lib().orc_cb_sweep_u(*args, int(uniforms)) if uniforms else lib().orc_cb_sweep(*args)
    if rc != OK:
        raise ValueError("oracle cb_sweep failed: %d" % rc)
    return obs, att.value, acc.value


def plane_uniform(seed, stream, sweep, colour, e):
    """The bit-plane uniform of colour-class site ``e`` (linear index >> 1)."""
    return lib().orc_plane_uniform(seed, stream, sweep, colour, e)


def bc_plane_bit(seed, stream, sweep, colour, e):
    """The Blume-Capel proposal bit of colour-class site ``e`` under bit-plane uniforms."""
    return int(lib().orc_bc_plane_bit(seed, stream, sweep, colour, e))


def seq_attempts(s, model, L, alg, beta, seed, stream=0, attempt0=0, nattempts=1, J=1.0, D=0.0, h=0.0):
    dim, Lv = _dims(L)
    st, ac = C.c_uint64(0), C.c_uint64(0)
    rc = lib().orc_seq_attempts(s, model, dim, Lv, alg, beta, J, D, h, seed, stream, attempt0, nattempts,
                                C.byref(st), C.byref(ac))
    if rc != OK:
        raise ValueError("oracle seq_attempts failed: %d" % rc)
    return st.value, ac.value


def flathist_sweep(s, model, L, mode, lnw, H, start, step, logf, seed, stream=0, sweep0=0, nsweeps=1,
                   J=1.0, D=0.0, h=0.0, record=True):
    """Returns (rc, obs, steps, accepted); lnw/H/s are updated in place."""
    dim, Lv = _dims(L)
    obs = np.zeros((nsweeps, 3), np.int64) if record else None
    st, ac = C.c_uint64(0), C.c_uint64(0)
    rc = lib().orc_flathist_sweep(s, model, dim, Lv, J, D, h, mode, lnw, H, start, step, len(lnw), logf,
                                  seed, stream, sweep0, nsweeps, obs.ctypes.data if record else None,
                                  C.byref(st), C.byref(ac))
    return rc, obs, st.value, ac.value


def flathist_trace(s, model, L, mode, lnw, H, start, step, logf, seed, stream=0, sweep0=0, nsweeps=1,
                   J=1.0, D=0.0, h=0.0):
    """flathist_sweep that also returns the (U, lr) of every decision in order:
    (rc, U[n], lr[n])."""
    dim, Lv = _dims(L)
    cap = int(np.prod(L)) * nsweeps
    u = np.zeros(cap, np.float64)
    lr = np.zeros(cap, np.float64)
    n = C.c_int64(0)
    rc = lib().orc_flathist_trace(s, model, dim, Lv, J, D, h, mode, lnw, H, start, step, len(lnw), logf, seed,
                                  stream, sweep0, nsweeps, u, lr, cap, C.byref(n))
    return rc, u[:n.value], lr[:n.value]


def muca_update(lnw, H):
    lib().orc_muca_update(lnw, H, len(lnw))


def wl_flat(H, visited, flatness):
    r = C.c_double(0)
    f = lib().orc_wl_flat(np.ascontiguousarray(H, np.int64), np.ascontiguousarray(visited, np.uint8), len(H),
                          flatness, C.byref(r))
    return bool(f), r.value


def pt_exchange(betas, pos, stage, x, seed, ladder, t, steps, accepted):
    """One exchange stage; ``pos``, ``steps``, ``accepted`` update in place; returns the new stage."""
    st = C.c_int32(stage)
    rc = lib().orc_pt_exchange(len(betas), np.ascontiguousarray(betas, np.float64), pos, C.byref(st),
                               np.ascontiguousarray(x, np.float64), seed, ladder, t, steps, accepted)
    assert rc == OK
    return st.value


def exp(x):
    return float(lib().orc_exp(float(x)))


def logistic(x):
    return float(lib().orc_logistic(float(x)))


class Graph:
    """A neighbour list in CSR form for the graph oracle: ``rowptr`` (int64, n+1),
    ``col`` (int32), optional per-entry couplings ``Jv`` (float64, the IsingMatrix
    values) and per-site fields ``hv`` (float64)."""

    def __init__(self, rowptr, col, Jv=None, J=1.0, hv=None, h=0.0):
        self.rowptr = np.ascontiguousarray(rowptr, np.int64)
        self.col = np.ascontiguousarray(col, np.int32)
        self.n = len(self.rowptr) - 1
        self.Jv = None if Jv is None else np.ascontiguousarray(Jv, np.float64)
        self.hv = None if hv is None else np.ascontiguousarray(hv, np.float64)
        self.J, self.h = float(J), float(h)

    def _ptrs(self):
        return (None if self.Jv is None else self.Jv.ctypes.data, None if self.hv is None else self.hv.ctypes.data)


class BCGraph(Graph):
    """A Blume-Capel neighbour list for the oracle: Graph plus the crystal field D."""

    def __init__(self, rowptr, col, Jv=None, J=1.0, D=0.0, hv=None, h=0.0):
        super().__init__(rowptr, col, Jv=Jv, J=J, hv=hv, h=h)
        self.D = float(D)


def bcg_init_random(n, seed, stream=0):
    s = np.zeros(n, np.int8)
    lib().orc_bcg_init_random(s, n, seed, stream)
    return s


def bcg_delta_energy(g, s, v, s_new):
    jv, hv = g._ptrs()
    return float(lib().orc_bcg_delta_energy(np.ascontiguousarray(s, np.int8), v, int(s_new), g.rowptr, g.col, jv,
                                            g.J, g.D, hv, g.h))


def bcg_observables(g, s):
    jv, hv = g._ptrs()
    E, M = C.c_double(), C.c_int64()
    lib().orc_bcg_observables(np.ascontiguousarray(s, np.int8), g.n, g.rowptr, g.col, jv, g.J, g.D, hv, g.h,
                              C.byref(E), C.byref(M))
    return E.value, M.value


def bcg_sweep(g, s, alg, beta, seed, stream=0, sweep0=0, nsweeps=1):
    """Blume-Capel colour-class sweeps in place; returns (E[nsweeps], M[nsweeps], attempts, accepts)."""
    jv, hv = g._ptrs()
    E0, M0 = bcg_observables(g, s)
    E, M = C.c_double(E0), C.c_int64(M0)
    Es = np.zeros(nsweeps, np.float64)
    Ms = np.zeros(nsweeps, np.int64)
    att, acc = C.c_uint64(0), C.c_uint64(0)
    rc = lib().orc_bcg_sweep(s, g.n, g.rowptr, g.col, jv, g.J, g.D, hv, g.h, alg, beta, seed, stream, sweep0, nsweeps,
                             C.byref(E), C.byref(M), Es.ctypes.data, Ms.ctypes.data, C.byref(att), C.byref(acc))
    if rc != OK:
        raise ValueError("oracle bcg_sweep failed: %d" % rc)
    return Es, Ms, att.value, acc.value


def graph_colour(g):
    c = np.zeros(g.n, np.int32)
    ncol = lib().orc_graph_colour(g.n, g.rowptr, g.col, c)
    return c, ncol


def graph_init_random(n, seed, stream=0):
    s = np.zeros(n, np.int8)
    lib().orc_graph_init_random(s, n, seed, stream)
    return s


def graph_delta_energy(g, s, v):
    jv, hv = g._ptrs()
    return float(lib().orc_graph_delta_energy(np.ascontiguousarray(s, np.int8), v, g.rowptr, g.col, jv, g.J, hv,
                                              g.h))


def graph_observables(g, s):
    jv, hv = g._ptrs()
    E, M = C.c_double(), C.c_int64()
    lib().orc_graph_observables(np.ascontiguousarray(s, np.int8), g.n, g.rowptr, g.col, jv, g.J, hv, g.h,
                                C.byref(E), C.byref(M))
    return E.value, M.value


def graph_sweep(g, s, alg, beta, seed, stream=0, sweep0=0, nsweeps=1):
    """Colour-class sweeps in place on ``s``; returns (E[nsweeps], M[nsweeps], attempts, accepts)
    with E and M the cached observables tracked from a full recompute before the first sweep."""
    jv, hv = g._ptrs()
    E0, M0 = graph_observables(g, s)
    E, M = C.c_double(E0), C.c_int64(M0)
    Es = np.zeros(nsweeps, np.float64)
    Ms = np.zeros(nsweeps, np.int64)
    att, acc = C.c_uint64(0), C.c_uint64(0)
    rc = lib().orc_graph_sweep(s, g.n, g.rowptr, g.col, jv, g.J, hv, g.h, alg, beta, seed, stream, sweep0, nsweeps,
                               C.byref(E), C.byref(M), Es.ctypes.data, Ms.ctypes.data, C.byref(att), C.byref(acc))
    if rc != OK:
        raise ValueError("oracle graph_sweep failed: %d" % rc)
    return Es, Ms, att.value, acc.value


def graph_seq_attempts(g, s, alg, beta, seed, stream=0, attempt0=0, nattempts=1):
    """nattempts random-site spin flips in place on ``s`` (Ising or, for a BCGraph,
    Blume-Capel rules); returns (E, M, attempts, accepts), E and M tracked from a full
    recompute before the first attempt."""
    jv, hv = g._ptrs()
    bc = isinstance(g, BCGraph)
    E0, M0 = bcg_observables(g, s) if bc else graph_observables(g, s)
    E, M = C.c_double(E0), C.c_int64(M0)
    att, acc = C.c_uint64(0), C.c_uint64(0)
    rc = lib().orc_graph_seq_attempts(s, g.n, g.rowptr, g.col, jv, g.J, hv, g.h, int(bc), g.D if bc else 0.0, alg,
                                      beta, seed, stream, attempt0, nattempts, C.byref(E), C.byref(M), C.byref(att),
                                      C.byref(acc))
    if rc != OK:
        raise ValueError("oracle graph_seq_attempts failed: %d" % rc)
    return E.value, M.value, att.value, acc.value


def tau_int(x, max_lag=None, c=5.0):
    """integrated_autocorrelation_time (src/measurements/autocorrelations.jl:28-67);
    raises ValueError where the reference raises ArgumentError."""
    x = np.ascontiguousarray(x, np.float64)
    v = lib().orc_tau_int(x, x.size, 0 if max_lag is None else int(max_lag), float(c))
    if v < 0:
        raise ValueError("invalid arguments")
    return float(v)


def bench_seq(model, L, alg, beta, seed, nthreads, attempts_per_thread, J=1.0, D=0.0, h=0.0):
    dim, Lv = _dims(L)
    sec = C.c_double(0)
    rc = lib().orc_bench_seq(model, dim, Lv, alg, beta, J, D, h, seed, nthreads, attempts_per_thread,
                             C.byref(sec))
    assert rc == OK
    return sec.value


__all__ = [n for n in dir() if not n.startswith("_")]

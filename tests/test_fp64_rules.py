"""How far the device's FP64 decisions are from the reference's literal arithmetic (CPU).

The flat-histogram and replica-exchange decisions are taken, on the device and in the
oracle alike, as ``lr > 0 || log(U) < lr`` with the project's own log (identical bits on
host and device).  The reference writes ``lr > 0 || rand(rng) < exp(lr)``
(src/algorithms/importance_sampling.jl:80-85, src/algorithms/replica_exchange.jl:115) and
its Multicanonical update ``lnw[b] -= log(h[b])`` (src/ensembles/multicanonical.jl:37-41)
with the language's own exp and log.  The two rules can only disagree when U lies within a
few ulps of exp(lr); these tests replay real decision streams of the configured
Blume-Capel L=1024 walkers (4,194,305 bins) and count the disagreements, and bound the
project log's error against the C library's log over every histogram count up to 2^24.
"""
import math

import numpy as np
import pytest

import oracle as O

L = [1024, 1024]
N = L[0] * L[1]
START, STEP, NB = -N, 1, 4 * N + 1


def _rules(U, lr):
    """(the device's log-domain rule, the reference's rule with numpy's exp, the
    reference's rule with the C library's exp) for every decision."""
    log_rule = (lr > 0) | (O.log_array(U) < lr)
    np_rule = (lr > 0) | (U < np.exp(lr))
    libm = np.fromiter((math.exp(v) for v in lr.tolist()), np.float64, lr.size)
    libm_rule = (lr > 0) | (U < libm)
    return log_rule, np_rule, libm_rule


def _near_ties(U, lr, rel=2.0 ** -40):
    """Decisions whose U lies within a relative 2^-40 of exp(lr): the only ones where any
    two exp / log implementations within a few ulps of each other could disagree."""
    m = lr <= 0
    p = np.exp(lr[m])
    return int(np.count_nonzero(np.abs(U[m] - p) <= rel * p))


@pytest.mark.parametrize("stream", ["muca_curved_weights", "wang_landau_logf_1"])
def test_flat_histogram_decisions_match_the_literal_rule(stream):
    """One sweep (1,048,576 decisions) of a configured Blume-Capel walker: Multicanonical
    with smooth non-linear weights (so lr takes a continuum of values, as with a converged
    ln g), and a first Wang-Landau stage (ln f = 1).  Both rules take the same decision
    every time."""
    s = O.init_random(O.BC, L, 11, 0)
    E = START + STEP * np.arange(NB, dtype=np.float64)
    if stream == "muca_curved_weights":
        lnw = -0.35 * E - 1e-7 * E * E
        mode, logf = O.MUCA, 0.0
    else:
        lnw = np.zeros(NB)
        mode, logf = O.WL, 1.0
    H = np.zeros(NB, np.int64)
    rc, U, lr = O.flathist_trace(s, O.BC, L, mode, lnw, H, START, STEP, logf, 11, stream=0, nsweeps=1, D=1.0)
    assert rc == O.OK and U.size == N
    log_rule, np_rule, libm_rule = _rules(U, lr)
    assert int(np.count_nonzero(log_rule != np_rule)) == 0
    assert int(np.count_nonzero(log_rule != libm_rule)) == 0
    assert _near_ties(U, lr) == 0


def test_project_log_error_over_histogram_counts():
    """The Multicanonical update subtracts log(H) for every count H >= 1.  Over every
    integer count up to 2^24 the project's log is within 1 ulp of numpy's log, so one
    update moves ln g by at most 1 ulp of log(H) plus the rounding of the subtraction from
    the reference's value."""
    H = np.arange(1, (1 << 24) + 1, dtype=np.float64)
    mine = O.log_array(H)
    ref = np.log(H)
    ulp = np.spacing(np.abs(ref))
    ulp[ref == 0.0] = np.spacing(0.0)
    err = np.abs(mine - ref) / ulp
    assert float(err.max()) <= 1.0
    # a sample checked against the C library's log directly
    idx = np.random.default_rng(3).integers(0, H.size, 20000)
    for i in idx.tolist():
        assert abs(mine[i] - math.log(H[i])) <= math.ulp(math.log(H[i]))

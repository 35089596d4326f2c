"""Host-side analysis of the per-sweep series: binning error bars, Binder cumulant and
the exact 2-D Ising results they are checked against.

The reference keeps only an integrated autocorrelation time
(src/measurements/autocorrelations.jl:28-110); the binning analysis, the Binder
cumulant and Onsager's results are restated from the published formulas:
  binning:  Flyvbjerg & Petersen, J. Chem. Phys. 91, 461 (1989)
  Binder:   U4 = 1 - <m^4> / (3 <m^2>^2), Binder, Z. Phys. B 43, 119 (1981)
  Onsager:  energy per site u = -coth(2b) [1 + (2/pi)(2 tanh^2(2b) - 1) K(k)],
            k = 2 sinh(2b) / cosh^2(2b), K the complete elliptic integral of the first
            kind (Onsager, Phys. Rev. 65, 117 (1944));
            spontaneous magnetisation m = (1 - sinh(2b)^-4)^(1/8) for b > b_c
            (Yang, Phys. Rev. 85, 808 (1952)), b_c = ln(1 + sqrt 2) / 2.
  Kaufman:  the partition function of the finite m x n torus (Kaufman, Phys. Rev. 76,
            1232 (1949); in the form of Ferdinand & Fisher, Phys. Rev. 185, 832 (1969)):
            Z = 1/2 (2 sinh 2K)^(mn/2) (Z1 + Z2 + Z3 + Z4), K = beta J,
            Z1 = prod_r 2 cosh(m g_{2r+1} / 2), Z2 = prod_r 2 sinh(m g_{2r+1} / 2),
            Z3 = prod_r 2 cosh(m g_{2r} / 2),   Z4 = prod_r 2 sinh(m g_{2r} / 2),
            r = 0 .. n-1, cosh g_l = cosh 2K coth 2K - cos(pi l / n) for l >= 1 and
            g_0 = 2K + ln tanh K (negative below the critical coupling).
"""
import math

import numpy as np

__all__ = ["binning_error", "binned_mean", "binder_cumulant", "jackknife", "onsager_energy_per_site",
           "onsager_magnetization", "BETA_C", "log_sum", "distribution_from_logdos", "kaufman_ising2d"]

BETA_C = 0.5 * math.log(1.0 + math.sqrt(2.0))


def binned_mean(x, nbins=32):
    """Mean and its error from `nbins` non-overlapping bins of the time series."""
    x = np.asarray(x, np.float64)
    n = len(x) // nbins * nbins
    if n == 0:
        raise ValueError("series shorter than the number of bins")
    b = x[:n].reshape(nbins, -1).mean(axis=1)
    return float(b.mean()), float(b.std(ddof=1) / math.sqrt(nbins))


def binning_error(x, min_bins=32):
    """Error of the mean from the binning analysis: the plateau of the naive error of
    bin means as the bin length doubles (largest value over bin lengths that leave at
    least `min_bins` bins)."""
    x = np.asarray(x, np.float64)
    best = 0.0
    L = 1
    while len(x) // L >= min_bins:
        n = len(x) // L
        b = x[: n * L].reshape(n, L).mean(axis=1)
        best = max(best, float(b.std(ddof=1) / math.sqrt(n)))
        L *= 2
    return best


def jackknife(f, cols, nbins=32):
    """Jackknife estimate and error of f(means of cols) over `nbins` blocks."""
    cols = [np.asarray(c, np.float64) for c in cols]
    n = len(cols[0]) // nbins * nbins
    blocks = [c[:n].reshape(nbins, -1) for c in cols]
    sums = [b.sum(axis=1) for b in blocks]
    tot = [s.sum() for s in sums]
    m = n // nbins
    full = f(*[t / n for t in tot])
    vals = np.array([f(*[(t - s[i]) / (n - m) for t, s in zip(tot, sums)]) for i in range(nbins)])
    err = math.sqrt((nbins - 1) / nbins * float(((vals - vals.mean()) ** 2).sum()))
    return float(full), err


def binder_cumulant(m, nbins=32):
    """U4 = 1 - <m^4> / (3 <m^2>^2) of the magnetisation series, with a jackknife error."""
    m = np.asarray(m, np.float64)
    return jackknife(lambda m2, m4: 1.0 - m4 / (3.0 * m2 * m2), [m ** 2, m ** 4], nbins)


def onsager_energy_per_site(beta, J=1.0):
    from scipy.special import ellipk
    b = beta * J
    k = 2.0 * math.sinh(2 * b) / math.cosh(2 * b) ** 2
    K = float(ellipk(k * k))
    return -J / math.tanh(2 * b) * (1.0 + (2.0 / math.pi) * (2.0 * math.tanh(2 * b) ** 2 - 1.0) * K)


def onsager_magnetization(beta, J=1.0):
    b = beta * J
    if b <= BETA_C:
        return 0.0
    return (1.0 - math.sinh(2 * b) ** -4) ** 0.125


def kaufman_ising2d(m, n, beta, J=1.0):
    """Exact (log Z, <E>) of the 2-D Ising model with coupling J on the periodic m x n
    lattice at inverse temperature beta, E = -J sum over the 2mn bonds of s_i s_j, from
    Kaufman's partition function (formula in the module docstring).  <E> = -J d ln Z / dK
    is evaluated analytically; products are summed as logarithms with their signs, so any
    size works in FP64.  m, n >= 3, beta J > 0."""
    m, n = int(m), int(n)
    if m < 3 or n < 3:
        raise ValueError("m, n >= 3")
    K = float(beta) * float(J)
    if not K > 0:
        raise ValueError("beta * J must be positive")
    s2, c2 = math.sinh(2 * K), math.cosh(2 * K)
    c = c2 * c2 / s2                                   # cosh 2K coth 2K
    dc = 2.0 * c2 * (s2 * s2 - 1.0) / (s2 * s2)        # d c / dK
    g = np.empty(2 * n)
    dg = np.empty(2 * n)
    g[0] = 2 * K + math.log(math.tanh(K))
    dg[0] = 2.0 + 2.0 / s2
    lv = np.arange(1, 2 * n)
    g[1:] = np.arccosh(c - np.cos(math.pi * lv / n))
    dg[1:] = dc / np.sinh(g[1:])
    x = 0.5 * m * g
    dx = 0.5 * m * dg

    def lcosh(v):  # log(2 cosh v), stable for large |v|
        a = np.abs(v)
        return a + np.log1p(np.exp(-2.0 * a))

    def lsinh(v):  # log|2 sinh v| for v != 0
        a = np.abs(v)
        return a + np.log1p(-np.exp(-2.0 * a))

    terms = []  # (log|Z_i| or None for an exact zero, sign, numerator of d ln Z contribution as (log, sign))
    for parity, kind in ((1, "cosh"), (1, "sinh"), (0, "cosh"), (0, "sinh")):
        xs, ds = x[parity::2], dx[parity::2]
        if kind == "cosh":
            lz = float(lcosh(xs).sum())
            d = float((ds * np.tanh(xs)).sum())
            terms.append((lz, 1.0, d, None))
            continue
        if np.all(xs != 0):
            lz = float(lsinh(xs).sum())
            sign = float(np.prod(np.sign(xs)))
            d = float((ds / np.tanh(xs)).sum())
            terms.append((lz, sign, d, None))
        else:  # g_0 = 0 exactly: the term vanishes, its derivative does not
            k = int(np.flatnonzero(xs == 0)[0])
            rest = np.delete(np.arange(xs.size), k)
            lrest = float(lsinh(xs[rest]).sum())
            terms.append((None, 0.0, 0.0, (lrest + math.log(2.0 * abs(ds[k])), float(np.sign(ds[k])))))
    top = max(t[0] for t in terms if t[0] is not None)
    den = sum(sg * math.exp(lz - top) for lz, sg, _, _ in terms if lz is not None)
    num = sum(sg * math.exp(lz - top) * d for lz, sg, d, _ in terms if lz is not None)
    num += sum(z[1] * math.exp(z[0] - top) for _, _, _, z in terms if z is not None)
    logz = math.log(0.5) + 0.5 * m * n * math.log(2.0 * s2) + top + math.log(den)
    dlogz = m * n * c2 / s2 + num / den
    return logz, -float(J) * dlogz


def log_sum(values):
    """log(sum(exp(values))) reduced pairwise as the reference's log_sum
    (src/infrastructure/utils.jl:54-73): c = max + log1p(exp(min - max))."""
    vals = [float(v) for v in values]
    if not vals:
        raise ValueError("values must be non-empty")
    acc = vals[0]
    for b in vals[1:]:
        a = acc
        acc = a + math.log1p(math.exp(b - a)) if a > b else b + math.log1p(math.exp(a - b))
    return acc


def distribution_from_logdos(centers, logdos, beta):
    """Canonical distribution at beta from a log density of states: reweight with
    exp(-beta E) over the finite entries and normalise (reweighting,
    src/infrastructure/utils.jl:95-105).  Entries that are not finite get 0."""
    E = np.asarray(centers, np.float64)
    lw = np.asarray(logdos, np.float64) - beta * E
    mask = np.isfinite(lw)
    if not mask.any():
        raise ValueError("logdos must contain at least one finite entry")
    lz = log_sum(lw[mask])
    out = np.zeros_like(lw)
    out[mask] = np.exp(lw[mask] - lz)
    return out

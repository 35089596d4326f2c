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
"""
import math

import numpy as np

__all__ = ["binning_error", "binned_mean", "binder_cumulant", "jackknife", "onsager_energy_per_site",
           "onsager_magnetization", "BETA_C", "log_sum", "distribution_from_logdos"]

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

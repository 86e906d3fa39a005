"""Error bars of a run's measurement series.

The engine records, per measurement (``record_series=True``), the energy per
site e, the magnetisation M of the reference's M^2 / M^4 accumulators, the
renormalised (block-spin) energy e_r and the correlated-pair product
<s_i.s_j>: the four columns of ``extras["series"]``.  Consecutive
measurements of a Markov chain are correlated, so the naive standard error of
a mean is too small by sqrt(2 tau_int).  This module gives

* ``binning``: the blocking analysis of Flyvbjerg and Petersen (J. Chem. Phys.
  91, 461 (1989)): the standard error of the mean of block averages for block
  sizes 1, 2, 4, ...; it rises with the block size and levels off once blocks
  are longer than the correlation time;
* ``tau_int``: the integrated autocorrelation time
  tau(W) = 1/2 + sum_{t=1..W} rho(t) with Sokal's automatic window (the
  smallest W with W >= c tau(W), c = 6);
* ``mean_error``: the mean with its binned error (the largest block size that
  leaves at least ``min_blocks`` blocks) and tau_int;
* ``jackknife``: mean and error of a function of several series' means over
  contiguous blocks (for C, chi and U4, which are not linear in the samples);
* ``summarize``: all of the above for an engine series.

Units are those of the series: energies per site in units of the couplings
handed to the engine (the reference divides them by T, mcMain.py:26-31), so the
specific heat is C = N var(e) and the susceptibility chi T = N (<M^2> - <|M|>^2).
"""
from __future__ import annotations

import numpy as np

SERIES_COLUMNS = ("e", "M", "e_r", "sij")


def binning(x, min_blocks: int = 32):
    """Block sizes 1, 2, 4, ... (while at least min_blocks blocks remain) and
    the standard error of the mean estimated from the block averages."""
    x = np.asarray(x, dtype=np.float64)
    sizes, errs = [], []
    b = 1
    while len(x) // b >= min_blocks:
        nb = len(x) // b
        blocks = x[: nb * b].reshape(nb, b).mean(axis=1)
        sizes.append(b)
        errs.append(float(blocks.std(ddof=1) / np.sqrt(nb)))
        b *= 2
    return np.array(sizes), np.array(errs)


def autocorrelation(x):
    """Normalised autocorrelation function rho(t), t = 0..n-1 (FFT, biased
    estimator: lag-t sums divided by n)."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    d = x - x.mean()
    var = float(np.dot(d, d)) / n
    if n < 2 or var == 0.0:
        return np.concatenate([[1.0], np.zeros(max(0, n - 1))])
    f = np.fft.rfft(d, 2 * n)
    acf = np.fft.irfft(f * np.conj(f))[:n] / n
    return acf / var


def tau_int(x, c: float = 6.0) -> float:
    """Integrated autocorrelation time with Sokal's automatic window."""
    rho = autocorrelation(x)
    tau = 0.5
    for w in range(1, len(rho)):
        tau += rho[w]
        if w >= c * tau:
            break
    return float(max(tau, 0.5))


def mean_error(x, min_blocks: int = 32):
    """(mean, binned error, tau_int).  The binned error is the one of the
    largest block size that keeps at least min_blocks blocks (the plateau of
    the blocking analysis when the run is long compared with tau_int)."""
    x = np.asarray(x, dtype=np.float64)
    _, errs = binning(x, min_blocks)
    err = float(errs[-1]) if len(errs) else float("nan")
    return float(x.mean()), err, tau_int(x)


def jackknife(fn, *series, nblocks: int = 32):
    """Mean and error of fn(mean(series_1), mean(series_2), ...) by the
    delete-one-block jackknife over nblocks contiguous blocks."""
    cols = [np.asarray(s, dtype=np.float64) for s in series]
    n = min(len(c) for c in cols)
    nb = min(nblocks, n)
    b = n // nb
    sums = [c[: nb * b].reshape(nb, b).sum(axis=1) for c in cols]
    tot = [s.sum() for s in sums]
    full = fn(*[t / (nb * b) for t in tot])
    reps = np.array([fn(*[(t - s[k]) / ((nb - 1) * b) for t, s in zip(tot, sums)]) for k in range(nb)])
    err = float(np.sqrt((nb - 1) / nb * ((reps - reps.mean()) ** 2).sum()))
    return float(full), err


def summarize(series, n_sites: int, min_blocks: int = 32):
    """Means with binned errors and tau_int of the four series columns and of
    e^2, |M|, M^2, M^4; jackknife values and errors of the specific heat
    C = N var(e), of chi T = N (<M^2> - <|M|>^2) and of the reference's
    U4 = <M^2>^2 / <M^4>.  Returns {name: (value, error, tau_int or None)}."""
    s = np.asarray(series, dtype=np.float64)
    e, M, er, sij = s[:, 0], s[:, 1], s[:, 2], s[:, 3]
    out = {}
    for name, x in (("e", e), ("e2", e * e), ("absM", np.abs(M)), ("M2", M * M), ("M4", M ** 4), ("e_r", er),
                    ("sij", sij)):
        out[name] = mean_error(x, min_blocks)
    N = float(n_sites)
    out["C"] = jackknife(lambda a, b: N * (b - a * a), e, e * e, nblocks=min_blocks) + (None,)
    out["chiT"] = jackknife(lambda a, b: N * (b - a * a), np.abs(M), M * M, nblocks=min_blocks) + (None,)
    out["U4"] = jackknife(lambda a, b: a * a / b if b != 0 else float("nan"), M * M, M ** 4,
                          nblocks=min_blocks) + (None,)
    return out

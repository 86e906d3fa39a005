"""Error analysis of measurement series (CPU): binning, tau_int, jackknife.

An AR(1) process x_t = phi x_{t-1} + sqrt(1 - phi^2) eps_t has unit variance
and the exact integrated autocorrelation time tau = (1 + phi) / (2 (1 - phi)),
so the error of a mean of n samples is sqrt(2 tau / n).  The estimators must
recover both within their own statistical scatter.
"""
import numpy as np
import pytest

from mcsolver_gb300 import analysis as A


def ar1(phi, n, seed):
    rng = np.random.default_rng(seed)
    eps = rng.standard_normal(n)
    x = np.empty(n)
    x[0] = eps[0]
    a = np.sqrt(1 - phi * phi)
    for t in range(1, n):
        x[t] = phi * x[t - 1] + a * eps[t]
    return x


@pytest.mark.parametrize("phi", [0.0, 0.5, 0.9])
def test_tau_and_binned_error_of_ar1(phi):
    n = 2 ** 17
    tau_exact = (1 + phi) / (2 * (1 - phi))
    err_exact = np.sqrt(2 * tau_exact / n)
    taus, errs = [], []
    for seed in range(4):
        x = ar1(phi, n, seed)
        m, err, tau = A.mean_error(x)
        taus.append(tau)
        errs.append(err)
    assert np.mean(taus) == pytest.approx(tau_exact, rel=0.12, abs=0.03)
    assert np.mean(errs) == pytest.approx(err_exact, rel=0.2)


def test_binning_rises_to_a_plateau():
    x = ar1(0.95, 2 ** 16, 7)
    sizes, errs = A.binning(x)
    assert sizes[0] == 1 and np.all(np.diff(sizes) > 0)
    naive = x.std(ddof=1) / np.sqrt(len(x))
    assert errs[0] == pytest.approx(naive)
    assert errs[-1] > 4 * naive  # sqrt(2 tau) = sqrt(39) ~ 6.2 for phi = 0.95


def test_jackknife_of_a_linear_function_is_the_blocked_mean_error():
    x = ar1(0.3, 4096, 3)
    v, e = A.jackknife(lambda a: 2.0 * a, x, nblocks=32)
    b = x.reshape(32, -1).mean(axis=1)
    assert v == pytest.approx(2 * x.mean())
    assert e == pytest.approx(2 * b.std(ddof=1) / np.sqrt(32), rel=1e-9)


def test_summarize_columns_and_derived_quantities():
    rng = np.random.default_rng(1)
    n = 4096
    e = -1.0 + 0.1 * rng.standard_normal(n)
    M = 0.5 + 0.05 * rng.standard_normal(n)
    s = np.stack([e, M, 0.5 * e, 0.9 + 0 * e], axis=1)
    out = A.summarize(s, n_sites=100)
    assert out["e"][0] == pytest.approx(e.mean())
    assert out["C"][0] == pytest.approx(100 * e.var(), rel=1e-9)
    assert out["chiT"][0] == pytest.approx(100 * (np.mean(M * M) - np.mean(np.abs(M)) ** 2), rel=1e-9)
    assert out["U4"][0] == pytest.approx(np.mean(M * M) ** 2 / np.mean(M ** 4), rel=1e-12)
    assert out["sij"][1] == pytest.approx(0.0, abs=1e-12)
    for k in ("e", "C", "U4"):
        assert out[k][1] > 0

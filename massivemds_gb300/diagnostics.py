"""MCMC diagnostics: effective sample size and minimum ESS per second.

ESS uses Geyer's initial monotone sequence estimator (Geyer 1992, "Practical
Markov chain Monte Carlo", Statistical Science 7:473-483): autocorrelations
rho_t of the chain, pair sums Gamma_k = rho_2k + rho_2k+1 truncated at the first
non-positive one and made monotone non-increasing, tau = -1 + 2 sum Gamma_k,
ESS = n / tau.

The MDS posterior is invariant to rotations and reflections of the latent
configuration, so chains are summarised through invariant functionals: the
log-likelihood, the precision, distances between fixed pairs of locations and
norms of fixed locations.
"""
from __future__ import annotations

import numpy as np


def autocorrelation(x: np.ndarray) -> np.ndarray:
    """Sample autocorrelation of a 1-D chain (FFT, biased normalisation)."""
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    x = x - x.mean()
    var = np.dot(x, x) / n
    if var == 0.0:
        return np.ones(n)
    size = 1 << (2 * n - 1).bit_length()
    f = np.fft.rfft(x, size)
    acov = np.fft.irfft(f * np.conj(f), size)[:n] / n
    return acov / var


def ess(x: np.ndarray) -> float:
    """Effective sample size of a 1-D chain (initial monotone sequence)."""
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    if n < 4:
        return float(n)
    if np.all(x == x[0]):
        return float("nan")
    rho = autocorrelation(x)
    m = (n - 1) // 2
    gammas = rho[0:2 * m:2] + rho[1:2 * m:2]
    tau_sum = 0.0
    prev = np.inf
    for g in gammas:
        if g <= 0.0:
            break
        g = min(g, prev)  # monotone non-increasing
        tau_sum += g
        prev = g
    tau = -1.0 + 2.0 * tau_sum
    tau = max(tau, 1.0 / np.log10(max(n, 10)))  # guard against antithetic chains
    return float(n / tau)


def min_ess(columns: np.ndarray) -> tuple[float, int]:
    """Smallest ESS over the columns of a (draws x functionals) array, and its column."""
    values = [ess(columns[:, k]) for k in range(columns.shape[1])]
    values = [v if np.isfinite(v) else np.inf for v in values]
    k = int(np.argmin(values))
    return float(values[k]), k


def invariant_functionals(result, include_precision: bool = False) -> np.ndarray:
    """Draws x functionals: log-likelihood, traced pair distances and location norms
    (and the precision when it is sampled) from an HmcResult."""
    cols = [result.column("log_likelihood")[:, None], result.pair_distances, result.location_norms]
    if include_precision:
        cols.insert(1, result.column("precision")[:, None])
    return np.hstack(cols)


def mcse_mean(x: np.ndarray) -> float:
    """Monte Carlo standard error of the mean of a chain."""
    x = np.asarray(x, dtype=np.float64)
    e = ess(x)
    return float(np.std(x, ddof=1) / np.sqrt(e)) if np.isfinite(e) and e > 0 else float("nan")

"""Integrated autocorrelation times of Monte Carlo series (no counterpart in
the reference, which reports plain means and variances).

tau_int = 1/2 + sum_{t>=1} rho(t), so that the variance of an N-sample mean is
2 tau_int var(x) / N and a series of N sweeps holds N / (2 tau_int)
effectively independent samples.  The sum is cut at the Madras-Sokal
automatic window: the smallest M with M >= c * tau_int(M) (Madras & Sokal,
J. Stat. Phys. 50, 109 (1988); c = 6 by default), and its statistical error is
their estimate tau * sqrt(2 (2M + 1) / N_total).
"""
from __future__ import annotations

from typing import Dict

import numpy as np


def autocovariance(series: np.ndarray) -> np.ndarray:
    """Mean autocovariance over replicas: series is [R, N] (or [N]); each row is
    centred on its own mean; returns C(t) for t = 0..N-1 (biased estimator, the
    usual one for windowed sums)."""
    x = np.atleast_2d(np.asarray(series, np.float64))
    R, N = x.shape
    x = x - x.mean(axis=1, keepdims=True)
    nfft = 1 << int(np.ceil(np.log2(2 * N)))
    f = np.fft.rfft(x, nfft, axis=1)
    acf = np.fft.irfft(f * np.conj(f), nfft, axis=1)[:, :N] / N
    return acf.mean(axis=0)


def tau_int(series: np.ndarray, c: float = 6.0) -> Dict[str, float]:
    """Madras-Sokal windowed integrated autocorrelation time of an [R, N]
    series set (R independent replicas of the same chain).  Returns tau, the
    window M, the error estimate, and whether the window closed before N/4 (a
    series shorter than that is too short for a reliable tau)."""
    x = np.atleast_2d(np.asarray(series, np.float64))
    R, N = x.shape
    C = autocovariance(x)
    if C[0] <= 0:
        return {"tau": 0.5, "window": 0, "err": 0.0, "reliable": True}
    rho = C / C[0]
    cum = 0.5 + np.cumsum(rho[1:])  # tau(M) for M = 1..N-1
    M = np.arange(1, N)
    ok = np.nonzero(M >= c * cum)[0]
    if len(ok) == 0:
        m = N - 1
        tau = float(cum[-1])
        reliable = False
    else:
        m = int(M[ok[0]])
        tau = float(cum[ok[0]])
        reliable = m < N // 4
    tau = max(tau, 0.5)
    err = tau * np.sqrt(2.0 * (2 * m + 1) / (R * N))
    return {"tau": tau, "window": m, "err": float(err), "reliable": bool(reliable)}


def ar1(n: int, phi: float, rng: np.random.Generator, replicas: int = 1) -> np.ndarray:
    """AR(1) series x_t = phi x_{t-1} + e_t started in equilibrium; its
    tau_int is (1 + phi) / (2 (1 - phi)).  Used to check the estimator."""
    x = np.empty((replicas, n))
    x[:, 0] = rng.normal(size=replicas) / np.sqrt(1 - phi * phi)
    e = rng.normal(size=(replicas, n))
    for t in range(1, n):
        x[:, t] = phi * x[:, t - 1] + e[:, t]
    return x

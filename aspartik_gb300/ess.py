"""Effective sample size of an MCMC trace.

Geyer's initial monotone sequence estimator (C. J. Geyer, "Practical Markov
chain Monte Carlo", Statistical Science 7(4), 1992): autocovariances are
summed in adjacent pairs Gamma_k = gamma_2k + gamma_2k+1 while the pairs stay
positive, each pair is lowered to the minimum of the pairs before it
(monotone), and tau = -1 + 2 sum_k Gamma_k / gamma_0.  ESS = n / tau.
"""

from __future__ import annotations

import numpy as np


def autocovariance(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    x = x - x.mean()
    size = 1 << (2 * n - 1).bit_length()
    f = np.fft.rfft(x, size)
    return np.fft.irfft(f * np.conj(f), size)[:n] / n


def ess(x, burn_in: float = 0.1) -> float:
    """ESS of a trace after discarding the first ``burn_in`` fraction."""
    x = np.asarray(x, dtype=np.float64)
    x = x[int(burn_in * x.size):]
    n = x.size
    if n < 4:
        return float(n)
    g = autocovariance(x)
    if g[0] <= 0.0:
        return float(n)
    pairs = g[: (n // 2) * 2].reshape(-1, 2).sum(axis=1)
    total = 0.0
    running_min = np.inf
    for gk in pairs:
        if gk <= 0.0:
            break
        running_min = min(running_min, gk)
        total += running_min
    tau = -1.0 + 2.0 * total / g[0]
    return float(n / max(tau, 1e-12))


def min_ess(traces: dict, burn_in: float = 0.1) -> tuple[float, dict]:
    per = {k: ess(v, burn_in) for k, v in traces.items()}
    return min(per.values()), per

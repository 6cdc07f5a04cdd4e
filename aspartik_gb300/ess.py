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


def multi_chain_ess(chains, burn_in: float = 0.1) -> float:
    """ESS of one scalar over m chains (A. Gelman et al., Bayesian Data
    Analysis, 3rd ed., 2013, sec. 11.5, in the form of the Stan reference
    manual): with W the mean within-chain variance, B/n the variance of the
    chain means and var+ = (n - 1)/n W + B/n, the combined autocorrelation is
    rho_t = 1 - (W - mean_j s_j^2 rho_t,j) / var+; Geyer's initial monotone
    sequence over rho gives tau and ESS = m n / tau.  Chains that disagree
    raise B, hence rho, so their ESS falls below the sum of the per-chain
    values; independent chains at stationarity give about that sum.  The
    first ``burn_in`` fraction of each chain is dropped and the chains are
    cut to a common length."""
    xs = [np.asarray(c, dtype=np.float64) for c in chains]
    xs = [x[int(burn_in * x.size):] for x in xs]
    n = min(x.size for x in xs)
    m = len(xs)
    if m == 1:
        return ess(xs[0], 0.0)
    if n < 4:
        return float(m * n)
    xs = [x[:n] for x in xs]
    acov = np.array([autocovariance(x) for x in xs]) * (n / (n - 1.0))  # s_j^2 rho_t,j
    w = acov[:, 0].mean()
    b_over_n = np.var([x.mean() for x in xs], ddof=1)
    var_plus = (n - 1.0) / n * w + b_over_n
    if var_plus <= 0.0:
        return float(m * n)
    rho = 1.0 - (w - acov.mean(axis=0)) / var_plus
    pairs = rho[: (n // 2) * 2].reshape(-1, 2).sum(axis=1)
    total = 0.0
    running_min = np.inf
    for pk in pairs:
        if pk <= 0.0:
            break
        running_min = min(running_min, pk)
        total += running_min
    tau = -1.0 + 2.0 * total
    return float(m * n / max(tau, 1e-12))

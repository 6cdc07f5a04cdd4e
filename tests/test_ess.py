"""ESS estimator (Geyer 1992 initial monotone sequence) on chains with a
known integrated autocorrelation time."""

import numpy as np
import pytest

from aspartik_gb300.ess import ess, min_ess


def ar1(n, rho, rng):
    x = np.empty(n)
    x[0] = rng.normal()
    e = rng.normal(size=n) * np.sqrt(1 - rho * rho)
    for i in range(1, n):
        x[i] = rho * x[i - 1] + e[i]
    return x


@pytest.mark.parametrize("rho", [0.0, 0.5, 0.9])
def test_ess_of_ar1_matches_theory(rho, rng):
    n = 200_000
    x = ar1(n, rho, rng)
    tau = (1 + rho) / (1 - rho)
    assert ess(x, burn_in=0.0) == pytest.approx(n / tau, rel=0.12)


def test_min_ess_picks_the_slowest_trace(rng):
    fast = rng.normal(size=50_000)
    slow = ar1(50_000, 0.95, rng)
    m, per = min_ess({"fast": fast, "slow": slow})
    assert m == per["slow"] < per["fast"]


def test_constant_and_short_traces():
    assert ess(np.ones(100)) == 90.0
    assert ess([1.0, 2.0]) == 2.0


@pytest.mark.parametrize("rho", [0.0, 0.9])
def test_multi_chain_ess_of_independent_chains_is_their_sum(rho, rng):
    """Stationary independent AR(1) chains: the combined ESS matches
    m n / tau, the sum of the per-chain values."""
    from aspartik_gb300.ess import multi_chain_ess

    m, n = 8, 40_000
    chains = [ar1(n, rho, rng) for _ in range(m)]
    tau = (1 + rho) / (1 - rho)
    assert multi_chain_ess(chains, burn_in=0.0) == pytest.approx(m * n / tau, rel=0.12)
    assert multi_chain_ess(chains, burn_in=0.0) == pytest.approx(
        sum(ess(c, burn_in=0.0) for c in chains), rel=0.1)


def test_multi_chain_ess_penalises_disagreeing_chains(rng):
    """Chains stuck around different means (not converged): each chain's own
    ESS is large, the combined ESS is far below their sum."""
    from aspartik_gb300.ess import multi_chain_ess

    chains = [ar1(5_000, 0.5, rng) + 3.0 * k for k in range(4)]
    summed = sum(ess(c, burn_in=0.0) for c in chains)
    assert multi_chain_ess(chains, burn_in=0.0) < 0.05 * summed


def test_multi_chain_ess_of_one_chain_is_its_ess(rng):
    from aspartik_gb300.ess import multi_chain_ess

    x = ar1(10_000, 0.7, rng)
    assert multi_chain_ess([x], burn_in=0.2) == ess(x, burn_in=0.2)

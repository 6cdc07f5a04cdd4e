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

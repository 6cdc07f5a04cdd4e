"""The native MCMC driver on the GPU: incremental likelihoods equal full
recomputes after thousands of proposals of every operator, the chain samples
the prior when the data carry no information, Metropolis coupling swaps, and
the FP32 chosen form and the FP64 plain form give the same posterior within
Monte Carlo error."""

import numpy as np
import pytest

from aspartik_gb300.ess import ess
from tests.cases import dna_case

pytestmark = pytest.mark.gpu


def make(case, **kw):
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    s = McmcSettings(**kw)
    m = Mcmc(case.leaves, case.weights, case.tree.parents, case.tree.heights, s)
    return m


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_every_operator_keeps_incremental_equal_to_full(precision):
    from aspartik_gb300.mcmc import OPERATORS

    c = dna_case(16, 300, seed=16, model="gtr", alpha=0.5, num_categories=4)
    weights = dict(tree_scale=3, subtree_slide=30, narrow_exchange=30, scale_alpha=1,
                   scale_birth_rate=3, delta_rates=1, delta_frequencies=1)
    m = make(c, model="gtr", precision=precision, num_categories=4, sample_every=10,
             weights=weights)
    m.set_parameters(rates=np.ones(6), frequencies=c.pi, alpha=0.5, birth_rate=2.0)
    for _ in range(6):
        m.run(500)
        assert m.check() < 1e-12
    stats = m.operator_stats()
    for name in weights:
        assert stats[name]["accepts"] > 0, name
    lnl = m.trace("lnl")
    assert lnl.size == 300 and np.isfinite(lnl).all()
    assert set(OPERATORS) == set(stats)


def test_flat_likelihood_samples_the_kappa_prior():
    """All tips unknown: the likelihood is constant, so ln(kappa) follows its
    LogNormal(1, 1.25) prior (config/__init__.py:706-708)."""
    c = dna_case(8, 50, seed=8)
    c.leaves = np.full_like(c.leaves, 0x0F)
    m = make(c, model="hky", precision="f64", num_categories=1, sample_every=5,
             weights=dict(scale_kappa=1.0), tune_every=500)
    m.set_parameters(kappa=2.0, frequencies=c.pi)
    m.run(60_000)
    assert abs(m.trace("lnl")).max() < 1e-9
    lk = np.log(m.trace("kappa_or_rate0"))[1000:]
    n_eff = ess(lk, burn_in=0.0)
    assert n_eff > 300
    se = 1.25 / np.sqrt(n_eff)
    assert abs(lk.mean() - 1.0) < 4.5 * se
    assert lk.std() == pytest.approx(1.25, rel=0.15)


def test_metropolis_coupling_swaps_and_stays_exact():
    c = dna_case(12, 200, seed=12, model="gtr")
    m = make(c, model="gtr", precision="f32", num_categories=1, num_chains=4, heat=0.1,
             swap_every=5, sample_every=10)
    m.set_parameters(rates=np.ones(6), frequencies=c.pi)
    m.run(2000)
    tried, accepted = m.swaps()
    assert tried == 400 and 0 < accepted <= tried
    assert m.check() < 1e-12
    betas = sorted(m.chain_state(i)[3] for i in range(4))
    assert betas == pytest.approx([1 / (1 + 0.1 * i) for i in (3, 2, 1, 0)])


def test_chosen_and_plain_forms_agree_on_the_posterior():
    """Same data, same moves: posterior means of the root height and kappa
    agree between the FP32 chosen form and the FP64 plain form within Monte
    Carlo error."""
    c = dna_case(16, 1000, seed=4, root_height=0.5)
    out = {}
    for precision, seed in (("f64", 11), ("f32", 12)):
        m = make(c, model="hky", precision=precision, num_categories=1, seed=seed,
                 sample_every=5, weights=dict(tree_scale=3, scale_kappa=1,
                                              subtree_slide=6, narrow_exchange=6))
        m.set_parameters(kappa=2.0, frequencies=c.pi)
        m.run(40_000)
        out[precision] = {k: m.trace(k)[800:] for k in ("root_height", "kappa_or_rate0")}
    for k in ("root_height", "kappa_or_rate0"):
        a, b = out["f64"][k], out["f32"][k]
        se = np.sqrt(a.var() / ess(a, 0.0) + b.var() / ess(b, 0.0))
        assert abs(a.mean() - b.mean()) < 5 * se, k


def test_chain_traces_of_independent_replicates():
    """Heat 0 without swaps runs independent replicates: every chain has a
    full trace of its own state, the reported cold chain is chain 0 (all at
    beta 1), the replicates' random streams differ, and each chain's lnL
    trace is its cached likelihood (incremental = full after the run)."""
    c = dna_case(16, 300, seed=18, model="gtr", alpha=0.5, num_categories=4)
    m = make(c, model="gtr", precision="f32", num_categories=4, num_chains=4, heat=0.0,
             swap_every=0, sample_every=10)
    m.set_parameters(rates=np.ones(6), frequencies=c.pi, alpha=0.5, birth_rate=2.0)
    m.run(2000)
    assert m.check() < 1e-12
    for name in ("lnl", "root_height", "kappa_or_rate0"):
        np.testing.assert_array_equal(m.trace(name, chain=0), m.trace(name))
        for k in range(4):
            assert m.trace(name, chain=k).size == 200
    lnl = [m.trace("lnl", chain=k) for k in range(4)]
    assert all(np.isfinite(t).all() for t in lnl)
    assert not np.array_equal(lnl[0], lnl[1])
    assert m.swaps() == (0, 0)
    from aspartik_gb300._native import B3GError

    with pytest.raises(B3GError):
        m.trace("lnl", chain=4)
    m.close()

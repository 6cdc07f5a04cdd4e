"""Relaxed clock (RelaxedClock, crates/b3/src/clock.rs:41-134) in the
native driver: category rates are median quantiles of a mean-one LogNormal;
the start likelihood equals the oracle's with per-edge scaled lengths; after
thousands of category and sd moves the incremental likelihood equals a full
recompute (a category change marks only its edge)."""

import ctypes as ct

import numpy as np
import pytest

from aspartik_gb300 import _native as nat
from oracle import oracle as O
from tests.cases import dna_case


def lognormal_categories(sd, k):
    out = np.zeros(k)
    nat.check(nat.lib.b3g_lognormal_categories(float(sd), k, nat.as_ptr(out, ct.c_double)))
    return out


@pytest.mark.parametrize("sd,k", [(0.05, 1), (0.3, 4), (1.0, 8), (2.5, 32)])
def test_lognormal_categories_match_scipy(sd, k):
    from scipy.stats import lognorm

    q = (np.arange(k) + 0.5) / k
    want = lognorm.ppf(q, s=sd, scale=np.exp(-0.5 * sd * sd))
    np.testing.assert_allclose(lognormal_categories(sd, k), want, rtol=1e-12)


def test_bad_category_arguments_are_rejected():
    out = np.zeros(4)
    assert nat.lib.b3g_lognormal_categories(0.0, 4, nat.as_ptr(out, ct.c_double)) != 0
    assert nat.lib.b3g_lognormal_categories(0.5, 0, nat.as_ptr(out, ct.c_double)) != 0


def relaxed_mcmc(c, precision, K, weights):
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    s = McmcSettings(model="gtr", precision=precision, num_categories=1, sample_every=10,
                     weights=weights, clock_categories=K, seed=9)
    return Mcmc(c.leaves, c.weights, c.tree.parents, c.tree.heights, s)


@pytest.mark.gpu
def test_start_likelihood_matches_oracle_with_edge_rates():
    c = dna_case(20, 400, seed=81, model="gtr")
    K, sd = 4, 0.6
    nodes = c.tree.parents.size
    cats = np.random.default_rng(3).integers(0, K, size=nodes).astype(np.uint32)
    m = relaxed_mcmc(c, "f64", K, dict(relaxed_category=1))
    m.set_clock(sd, cats)
    m.set_parameters(rates=c.rates, frequencies=c.pi, birth_rate=1.0)
    _, _, lnl, _ = m.chain_state(0)
    rates = lognormal_categories(sd, K)
    t = O.DatedTree(c.tree.parents, c.tree.heights)
    t.mark_all_edges_updated()
    internals, children = t.partials_lists()
    model = O.gtr(c.rates, c.pi)
    mats = np.array([[model.transition(t.edge_length(int(e)) * rates[cats[int(e)]])
                      for e in pair] for pair in children])
    calc = O.Cpu4Calculator(c.leaves, c.leaves.shape[1], 30, 1)
    calc.propose(internals, children, mats, c.pi)
    want = float(np.array(calc.likelihoods()) @ c.weights.astype(np.float64))
    assert lnl == pytest.approx(want, rel=1e-10)
    m.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 1e-12)])
def test_category_and_sd_moves_keep_incremental_equal_to_full(precision, tol):
    c = dna_case(24, 500, seed=82, model="gtr")
    weights = dict(relaxed_category=20, scale_clock_sd=3, subtree_slide=10,
                   narrow_exchange=10, tree_scale=1)
    m = relaxed_mcmc(c, precision, 6, weights)
    m.set_clock(0.4)
    m.set_parameters(rates=c.rates, frequencies=c.pi, birth_rate=1.0)
    for _ in range(5):
        m.run(400)
        assert m.check() < tol
    stats = m.operator_stats()
    assert stats["relaxed_category"]["accepts"] > 0
    assert stats["scale_clock_sd"]["accepts"] > 0
    sd = m.trace("clock_sd")
    assert sd.size == 200 and (sd > 0).all() and np.unique(sd).size > 1
    m.close()

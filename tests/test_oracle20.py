"""The generic-S oracle (oracle/generic.py) pinned before it checks the
20-state GPU path: it equals the 4-state cpu4 restatement at S = 4, the
JC-20 closed form, and brute-force enumeration at S = 20."""

import numpy as np
import pytest

from oracle import brute
from oracle import generic as G
from oracle import oracle as O
from tests.cases import dna_case, protein_case

_DNA_STATE = {1: 0, 2: 1, 4: 2, 8: 3}


def dna_states(leaves):
    out = np.full(leaves.shape, 4, dtype=np.uint8)
    for code, st in _DNA_STATE.items():
        out[leaves == code] = st
    return out


@pytest.mark.parametrize("alpha,K", [(None, 1), (0.5, 4)])
def test_generic_at_four_states_equals_cpu4(alpha, K):
    c = dna_case(24, 600, seed=5, model="gtr", alpha=alpha, num_categories=K, gaps=0.05,
                 ambiguous=0.02)
    model = O.gtr(c.rates, c.pi)
    t = O.DatedTree(c.tree.parents, c.tree.heights)
    if K == 1:
        ref = O.DnaLikelihood(c.leaves, c.weights, t, model).cache
    else:
        ref = O.GammaLikelihood(c.leaves, c.weights, t, model, K, alpha).cache
    cats = O.gamma_categories(alpha, K) if alpha else None
    got = G.log_likelihood(dna_states(c.leaves), c.weights, c.tree.parents, c.tree.heights,
                           model, cats)
    assert got == pytest.approx(ref, rel=1e-12)


def test_jc20_closed_form():
    """P_ii = 1/20 + 19/20 e^{-20t/19}, P_ij = 1/20 - 1/20 e^{-20t/19}."""
    m = O.reversible(np.ones(190), np.full(20, 0.05))
    for t in (1e-3, 0.1, 0.7, 3.0):
        P = m.transition(t)
        e = np.exp(-20.0 * t / 19.0)
        want = np.full((20, 20), 0.05 - 0.05 * e)
        np.fill_diagonal(want, 0.05 + 0.95 * e)
        # the eigen route loses ~1e-14 absolute to cancellation
        np.testing.assert_allclose(P, want, rtol=1e-12, atol=1e-13)


def test_twenty_states_equal_brute_force():
    rng = np.random.default_rng(20)
    c = protein_case(3, 40, seed=21, alpha=None, num_categories=1, gaps=0.1)
    model = O.reversible(c.rates, c.pi)
    site = G.site_log_likelihoods(c.leaves, c.tree.parents, c.tree.heights, model)
    want = brute.site_log_likelihoods(c.tree.parents, c.tree.heights, c.leaves,
                                      model.Q.reshape(20, 20), c.pi)
    np.testing.assert_allclose(site, np.asarray(want, dtype=np.float64), rtol=1e-11)
    # and with Gamma categories
    cats = O.gamma_categories(0.7, 3)
    site = G.site_log_likelihoods(c.leaves, c.tree.parents, c.tree.heights, model, cats)
    want = brute.site_log_likelihoods(c.tree.parents, c.tree.heights, c.leaves,
                                      model.Q.reshape(20, 20), c.pi, cat_rates=cats)
    np.testing.assert_allclose(site, np.asarray(want, dtype=np.float64), rtol=1e-11)
    assert rng is not None


def test_scale_invariance_at_twenty_states():
    c = protein_case(64, 300, seed=22, alpha=1.0, num_categories=4)
    model = O.reversible(c.rates, c.pi)
    cats = O.gamma_categories(1.0, 4)
    vals = [G.log_likelihood(c.leaves, c.weights, c.tree.parents, c.tree.heights, model,
                             cats, scale_ln=s) for s in (3, 30, 300)]
    assert vals[0] == pytest.approx(vals[1], rel=1e-12)
    assert vals[2] == pytest.approx(vals[1], rel=1e-12)

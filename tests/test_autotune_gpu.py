"""The autotuner picks a launch configuration and leaves the accepted state
unchanged: the next proposal gives the same likelihood as on a calculator
that was never tuned."""

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import dna_case, protein_case
from tests.test_gpu_parity import F32_TOL, lists_and_lengths, make_gpu
from tests.test_oracle import random_move

pytestmark = pytest.mark.gpu


def whole(tree):
    tree.mark_all_edges_updated()
    return lists_and_lengths(tree)


def test_dna_tile_choice_keeps_state(rng):
    c = dna_case(96, 3000, seed=61, model="gtr", alpha=0.5, num_categories=4)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    tuned, plain = make_gpu(c.leaves, c.weights, 4, "f32"), make_gpu(c.leaves, c.weights, 4, "f32")
    full = whole(tree)
    for g in (tuned, plain):
        g.set_reversible(c.rates, c.pi)
        g.set_gamma(0.5)
        g.propose_lengths(*full, 1.0)
        g.accept()
    tree.accept()
    choice = tuned.autotune(*full, 1.0)
    assert choice in (16, 32, 64, 128)
    for _ in range(4):
        random_move(tree, rng)
        inc = lists_and_lengths(tree)
        tuned.propose_lengths(*inc, 1.0)
        plain.propose_lengths(*inc, 1.0)
        a, b = tuned.log_likelihood(), plain.log_likelihood()
        np.testing.assert_array_equal(tuned.site_log_likelihoods(), plain.site_log_likelihoods())
        assert a == pytest.approx(b, rel=1e-12)
        tree.accept()
        tuned.accept()
        plain.accept()
    # whole tree again with the tuned tile
    tuned.propose_lengths(*whole(tree), 1.0)
    plain.propose_lengths(*whole(tree), 1.0)
    assert tuned.log_likelihood() == pytest.approx(plain.log_likelihood(), rel=1e-12)
    tuned.close()
    plain.close()


def test_twenty_state_engine_choice_keeps_state():
    from aspartik_gb300.calculator import Calculator

    c = protein_case(64, 1500, seed=62, alpha=1.0, num_categories=4)
    g = Calculator.GB300(0, "f32").make20(c.leaves, c.leaves.shape[1], num_categories=4)
    g.set_weights(c.weights)
    g.set_reversible(c.rates, c.pi)
    g.set_gamma(1.0)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    full = whole(tree)
    g.propose_lengths(*full, 1.0)
    before = g.log_likelihood()
    g.accept()
    assert g.autotune(*full, 1.0) in (0, 1)
    g.propose_lengths(*full, 1.0)
    assert g.log_likelihood() == pytest.approx(before, rel=F32_TOL)
    g.close()


def test_fp64_form_has_nothing_to_tune():
    c = dna_case(16, 200, seed=63)
    g = make_gpu(c.leaves, c.weights)
    m = O.hky(2.0, c.pi)
    g.set_eigen(m.V, m.Vinv, m.lam, m.Q, m.pi)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    assert g.autotune(*whole(tree), 1.0) == 0
    g.close()

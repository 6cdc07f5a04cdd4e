"""Batched evaluation: heterogeneous chains (taxa, sites, categories) in one
graph-replayed launch give the same log-likelihoods as evaluating each chain
on its own, through dirty-path proposals with accept and reject."""

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import dna_case

pytestmark = pytest.mark.gpu

SHAPES = [(24, 500, 4), (57, 3000, 4), (130, 1200, 1), (40, 20000, 2), (200, 800, 4),
          (33, 700, 8)]


def lists(tree: O.DatedTree):
    internals, children = tree.partials_lists()
    lengths = np.array([[tree.edge_length(int(a)), tree.edge_length(int(b))]
                        for a, b in children]).reshape(-1, 2)
    return internals, children, lengths


def build(shape, seed):
    from aspartik_gb300.calculator import Calculator

    L, N, K = shape
    c = dna_case(L, N, seed=seed, model="gtr", alpha=0.7 if K > 1 else None,
                 num_categories=K, root_height=1.0)
    calcs = []
    for _ in range(2):  # one batch member, one evaluated alone
        g = Calculator.GB300(0, "f32").make4(c.leaves, c.leaves.shape[1], num_categories=K)
        g.set_weights(c.weights)
        g.set_reversible(c.rates, c.pi)
        if K > 1:
            g.set_gamma(0.7)
        calcs.append(g)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    tree.mark_all_edges_updated()
    return c, tree, calcs[0], calcs[1]


def test_batch_matches_individual_evaluation(rng):
    from aspartik_gb300.calculator import Batch
    from tests.test_oracle import random_move

    probs = [build(s, 100 + i) for i, s in enumerate(SHAPES)]
    batch = Batch([p[2] for p in probs])
    for step in range(25):
        active = [True] * len(probs) if step == 0 else list(rng.random(len(probs)) < 0.8)
        for (c, tree, member, alone), act in zip(probs, active):
            if step and act:
                random_move(tree, rng)
            if act:
                args = lists(tree)
                member.stage_lengths(*args, 1.0)
                alone.propose_lengths(*args, 1.0)
        batch.run()
        got = batch.log_likelihoods()
        for k, ((c, tree, member, alone), act) in enumerate(zip(probs, active)):
            if not act:
                assert np.isnan(got[k])
                continue
            want = alone.log_likelihood()
            assert got[k] == pytest.approx(want, rel=1e-12), (step, k)
        for (c, tree, member, alone), act in zip(probs, active):
            if not act:
                continue
            if rng.random() < 0.5:
                tree.accept(); member.accept(); alone.accept()  # noqa: E702
            else:
                tree.reject(); member.reject(); alone.reject()  # noqa: E702
    assert batch.last_ms() > 0.0


def test_batch_membership_rules():
    from aspartik_gb300._native import B3G_ERR_INVALID_ARGUMENT, B3G_ERR_STATE, B3GError
    from aspartik_gb300.calculator import Batch, Calculator

    c = dna_case(10, 100, seed=1)
    f64 = Calculator.GB300(0, "f64").make4(c.leaves, c.leaves.shape[1])
    with pytest.raises(B3GError) as e:
        Batch([f64])
    assert e.value.status == B3G_ERR_INVALID_ARGUMENT
    f32 = Calculator.GB300(0, "f32").make4(c.leaves, c.leaves.shape[1])
    f32.set_reversible(np.ones(6), c.pi)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    tree.mark_all_edges_updated()
    with pytest.raises(B3GError) as e:
        f32.stage_lengths(*lists(tree))
    assert e.value.status == B3G_ERR_STATE
    b = Batch([f32])
    with pytest.raises(B3GError) as e:
        Batch([f32])
    assert e.value.status == B3G_ERR_INVALID_ARGUMENT
    f32.stage_lengths(*lists(tree))
    b.run()
    ref = O.DnaLikelihood(c.leaves, c.weights, O.DatedTree(c.tree.parents, c.tree.heights),
                          O.gtr(np.ones(6), c.pi)).cache
    # weights were not set on this calculator: every pattern counts once
    assert np.isfinite(b.log_likelihoods()[0])
    b.close()
    f32.set_weights(c.weights)
    f32.propose_lengths(*lists(tree))  # usable alone again after the batch
    assert f32.log_likelihood() == pytest.approx(ref, rel=1e-6)

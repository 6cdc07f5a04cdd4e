"""Per-pattern class mixture (HeteroLikelihood, likelihood/hetero.rs:97-168)
against the oracle: K classes with their own model and clock rate over the
same patterns, pattern p counted under class c(p)."""

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import dna_case
from tests.test_gpu_parity import F32_TOL, F64_TOL, lists_and_lengths, make_gpu
from tests.test_oracle import random_move

pytestmark = pytest.mark.gpu


def oracle_sites(c, tree, model, clock):
    """Per-pattern lnL of one class (one category) on the oracle."""
    t = O.DatedTree(np.array(tree.parents), np.array(tree.heights))
    t.mark_all_edges_updated()
    internals, children = t.partials_lists()
    mats = np.array([[model.transition(t.edge_length(int(x)) * clock) for x in pair]
                     for pair in children])
    calc = O.Cpu4Calculator(c.leaves, c.leaves.shape[1], 30, 1)
    calc.propose(internals, children, mats, model.frequencies())
    return np.array(calc.likelihoods())


def whole(tree):
    tree.mark_all_edges_updated()
    return lists_and_lengths(tree)


@pytest.mark.parametrize("precision,tol", [("f64", F64_TOL), ("f32", F32_TOL)])
def test_mixture_matches_oracle_through_steps(precision, tol, rng):
    from aspartik_gb300.calculator import Hetero

    c = dna_case(40, 1200, seed=71, model="gtr", gaps=0.02)
    P = c.leaves.shape[1]
    K = 3
    models = [O.gtr(c.rates, c.pi), O.hky(3.0, c.pi),
              O.gtr(rng.gamma(2.0, 1.0, 6), np.full(4, 0.25))]
    rates_of = [c.rates, None, None]
    clocks = [1.0, 0.6, 1.7]
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    members = []
    for k in range(K):
        g = make_gpu(c.leaves, c.weights, 1, precision)
        m = models[k]
        g.set_eigen(m.V, m.Vinv, m.lam, m.Q, m.pi)
        g.propose_lengths(*whole(tree), clocks[k])
        g.accept()
        members.append(g)
    tree.accept()
    mix = Hetero(members)

    def want(classes):
        sites = np.array([oracle_sites(c, tree, models[k], clocks[k]) for k in range(K)])
        return float(sites[classes, np.arange(P)] @ c.weights.astype(np.float64))

    cls = np.zeros(P, dtype=np.uint32)
    assert mix.log_likelihood() == pytest.approx(want(cls), rel=tol)
    mix.accept()
    for step in range(8):
        kind = step % 3
        if kind == 0:  # classes only: no pruning
            new = rng.integers(0, K, size=P).astype(np.uint32)
            mix.set_classes(new)
        elif kind == 1:  # tree move: every class re-evaluated
            random_move(tree, rng)
            inc = lists_and_lengths(tree)
            for k, g in enumerate(members):
                g.propose_lengths(*inc, clocks[k])
            new = cls
        else:  # both, only class 1's clock changes
            clocks_new = list(clocks)
            clocks_new[1] = clocks[1] * 1.1
            tree_copy = O.DatedTree(np.array(tree.parents), np.array(tree.heights))
            members[1].propose_lengths(*whole(tree_copy), clocks_new[1])
            new = rng.integers(0, K, size=P).astype(np.uint32)
            mix.set_classes(new)
        if kind == 2:
            saved = clocks[1]
            clocks[1] = clocks_new[1]
        got = mix.log_likelihood()
        assert got == pytest.approx(want(new), rel=tol), step
        if rng.random() < 0.5:
            mix.accept()
            tree.accept()
            cls = new
        else:
            mix.reject()
            tree.reject()
            if kind == 2:
                clocks[1] = saved
        # the accepted state is what the next classes-only step sees
        probe = rng.integers(0, K, size=P).astype(np.uint32)
        mix.set_classes(probe)
        assert mix.log_likelihood() == pytest.approx(want(probe), rel=tol), step
        mix.reject()
    mix.close()
    for g in members:
        g.close()


def test_mixture_rejects_bad_input():
    from aspartik_gb300.calculator import B3GError, Hetero

    c = dna_case(8, 100, seed=72)
    m = O.hky(2.0, c.pi)
    g = make_gpu(c.leaves, c.weights)
    g.set_eigen(m.V, m.Vinv, m.lam, m.Q, m.pi)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    with pytest.raises(B3GError):  # never evaluated
        Hetero([g])
    g.propose_lengths(*whole(tree), 1.0)
    with pytest.raises(B3GError):  # evaluated but not accepted
        Hetero([g])
    g.accept()
    mix = Hetero([g])
    with pytest.raises(B3GError):
        mix.set_classes(np.full(c.leaves.shape[1], 1, dtype=np.uint32))
    mix.close()
    g.close()

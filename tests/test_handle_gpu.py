"""Tree-level handle (b3g_create / b3g_set_tree / b3g_mark_edges /
b3g_propose / b3g_lnl / b3g_accept / b3g_reject) against the oracle: several
chains proposed together, each with its own moves, the library building the
dirty lists from its mirrored trees as partials_lists does
(tree.rs:357-461), accept/reject sequences, per-pattern values and the
errors of the interface."""

import numpy as np
import pytest

from aspartik_gb300._native import B3G_ERR_INVALID_ARGUMENT, B3G_ERR_STATE, B3GError
from oracle import oracle as O
from tests.cases import dna_case
from tests.test_gpu_parity import F32_TOL, F64_TOL
from tests.test_oracle import random_move

pytestmark = pytest.mark.gpu


def oracle_lnl(c, tree, model, K, alpha, clock):
    t = O.DatedTree(np.array(tree.parents), np.array(tree.heights))
    return O.GammaLikelihood(c.leaves, c.weights, t, model, K, alpha, clock_rate=clock).cache


def changed_edges(old_p, old_h, new_p, new_h):
    """Edges whose length or parent differ (edge id = child node id)."""
    out = []
    for v in range(len(new_p)):
        if new_p[v] == 0xFFFFFFFF:
            continue
        if (old_p[v] != new_p[v] or old_h[v] != new_h[v]
                or old_h[new_p[v]] != new_h[new_p[v]]):
            out.append(v)
    return out


@pytest.mark.parametrize("precision,tol", [("f64", F64_TOL), ("f32", F32_TOL)])
def test_chains_through_moves_match_oracle(precision, tol):
    from aspartik_gb300.handle import Handle

    K, alpha, chains = 4, 0.5, 3
    c = dna_case(40, 1500, seed=101, model="gtr", root_height=1.0, alpha=alpha,
                 num_categories=K, gaps=0.02)
    model = O.gtr(c.rates, c.pi)
    cats = O.gamma_categories(alpha, K)
    rng = np.random.default_rng(7)
    h = Handle(c.leaves, c.weights, chains, precision=precision, num_categories=K)
    trees, clocks = [], [1.0, 0.8, 1.3]
    for k in range(chains):
        t = O.DatedTree(c.tree.parents, c.tree.heights)
        trees.append(t)
        h.set_model(k, model.V, model.Vinv, model.lam, model.pi, cats)
        h.set_tree(k, np.array(t.parents), np.array(t.heights), clocks[k])
        h.mark_all(k)
    h.propose()
    h.wait()
    for k in range(chains):
        want = oracle_lnl(c, trees[k], model, K, alpha, clocks[k])
        assert h.lnl(k) == pytest.approx(want, rel=tol)
        h.accept(k)
        trees[k].accept()
    for step in range(12):
        for k in range(chains):
            old_p, old_h = np.array(trees[k].parents), np.array(trees[k].heights)
            for _ in range(1 + step % 3):
                random_move(trees[k], rng)
            new_p, new_h = np.array(trees[k].parents), np.array(trees[k].heights)
            h.set_tree(k, new_p, new_h, clocks[k])
            h.mark_edges(k, changed_edges(old_p, old_h, new_p, new_h))
        h.propose()  # all chains at once
        for k in range(chains):
            want = oracle_lnl(c, trees[k], model, K, alpha, clocks[k])
            assert h.lnl(k) == pytest.approx(want, rel=tol), (step, k)
            if rng.random() < 0.5:
                h.accept(k)
                trees[k].accept()
            else:
                h.reject(k)
                trees[k].reject()
    # a proposal on one chain only, per-pattern values summing to the total
    k = 1
    old_p, old_h = np.array(trees[k].parents), np.array(trees[k].heights)
    random_move(trees[k], rng)
    new_p, new_h = np.array(trees[k].parents), np.array(trees[k].heights)
    h.set_tree(k, new_p, new_h, clocks[k])
    h.mark_edges(k, changed_edges(old_p, old_h, new_p, new_h))
    h.propose([k])
    site = h.site_lnl(k)
    assert float(site @ c.weights.astype(np.float64)) == pytest.approx(h.lnl(k), rel=1e-12)
    assert h.lnl(k) == pytest.approx(oracle_lnl(c, trees[k], model, K, alpha, clocks[k]),
                                     rel=tol)
    h.close()


def test_errors_leave_the_handle_usable():
    from aspartik_gb300.handle import Handle

    c = dna_case(12, 300, seed=102, model="hky")
    model = O.hky(2.0, c.pi)
    h = Handle(c.leaves, c.weights, 2)
    h.set_model(0, model.V, model.Vinv, model.lam, model.pi, [1.0])
    with pytest.raises(B3GError) as e:
        h.propose([0])  # no tree yet
    assert e.value.status == B3G_ERR_STATE
    h.set_tree(0, c.tree.parents, c.tree.heights, 1.0)
    with pytest.raises(B3GError) as e:
        h.mark_edges(0, [2 * 12 - 2])  # the root has no edge
    assert e.value.status == B3G_ERR_INVALID_ARGUMENT
    with pytest.raises(B3GError) as e:
        h.propose([5])  # no such chain
    assert e.value.status == B3G_ERR_INVALID_ARGUMENT
    bad = np.array(c.tree.heights)
    bad[-1] = 0.0  # root below its children
    with pytest.raises(B3GError) as e:
        h.set_tree(0, c.tree.parents, bad, 1.0)
    assert e.value.status == B3G_ERR_INVALID_ARGUMENT
    with pytest.raises(ValueError):  # two category rates, one category
        h.set_model(0, model.V, model.Vinv, model.lam, model.pi, [0.5, 1.5])
    h.mark_all(0)
    h.propose([0])
    t = O.DatedTree(c.tree.parents, c.tree.heights)
    want = O.DnaLikelihood(c.leaves, c.weights, t, model).cache
    assert h.lnl(0) == pytest.approx(want, rel=F64_TOL)
    h.close()

"""The fused one-launch evaluation of short FP32 lists (schedule, lengths and
root frequencies as kernel parameters, transition tables built in shared
memory, result written to mapped host memory) against the two-kernel path
and the CPU oracle.

The two paths share the per-column arithmetic and build bit-identical
transition tables, so per-site log-likelihoods must agree exactly; the total
may differ in the last bits only through the order of the tile sums (the
two-kernel path uses 64-pattern tiles for lists that are not path-like).
"""

import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import dna_case
from tests.test_gpu_parity import F32_TOL, full, lists_and_lengths, make_gpu
from tests.test_oracle import random_move

pytestmark = pytest.mark.gpu


def make_pair(c, K, alpha):
    """(fused, two-kernel) FP32 calculators on the same data and model."""
    old = os.environ.get("B3G_DIRECT")
    try:
        os.environ["B3G_DIRECT"] = "0"
        two = make_gpu(c.leaves, c.weights, K, "f32")
    finally:
        if old is None:
            os.environ.pop("B3G_DIRECT", None)
        else:
            os.environ["B3G_DIRECT"] = old
    fused = make_gpu(c.leaves, c.weights, K, "f32")
    for g in (fused, two):
        g.set_reversible(c.rates, c.pi)
        g.set_gamma(alpha)
    return fused, two


@pytest.mark.parametrize("K", [4, 2, 1])
def test_short_lists_match_two_kernel_path_and_oracle(rng, K):
    c = dna_case(64, 3000, seed=91, model="gtr", alpha=0.5, num_categories=K, gaps=0.02)
    fused, two = make_pair(c, K, 0.5)
    fused.set_timing(True)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    ref = O.GammaLikelihood(c.leaves, c.weights, tree, O.gtr(c.rates, c.pi), K, 0.5)
    tree.mark_all_edges_updated()
    for g in (fused, two):  # 63 entries: both take the two-kernel path
        g.propose_lengths(*lists_and_lengths(tree), 1.0)
        g.accept()
    ref.likelihood()
    tree.accept()
    ref.accept()
    for step in range(40):
        random_move(tree, rng)
        internals, children, lengths = lists_and_lengths(tree)
        assert 0 < len(internals) <= 48
        want = ref.likelihood()
        fused.propose_lengths(internals, children, lengths, 1.0)
        two.propose_lengths(internals, children, lengths, 1.0)
        a, b = fused.log_likelihood(), two.log_likelihood()
        assert a == pytest.approx(want, rel=F32_TOL), step
        assert a == pytest.approx(b, rel=1e-12, abs=0.0), step
        np.testing.assert_array_equal(fused.site_log_likelihoods(),
                                      two.site_log_likelihoods())
        t, p = fused.last_timing()
        assert t == 0.0 and p > 0.0  # one fused kernel
        if rng.random() < 0.5:
            tree.accept(); ref.accept()  # noqa: E702
            fused.accept(); two.accept()  # noqa: E702
        else:
            tree.reject(); ref.reject()  # noqa: E702
            fused.reject(); two.reject()  # noqa: E702
    fused.close()
    two.close()


def test_interleaved_paths_read_listed_children_from_memory(rng):
    """Several height changes in different subtrees: the list interleaves
    paths, so some listed children are neither of the two previous entries
    and come back from memory."""
    c = dna_case(96, 1500, seed=17, model="gtr", alpha=1.0, num_categories=4)
    fused, two = make_pair(c, 4, 1.0)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    ref = O.GammaLikelihood(c.leaves, c.weights, tree, O.gtr(c.rates, c.pi), 4, 1.0)
    tree.mark_all_edges_updated()
    for g in (fused, two):
        g.propose_lengths(*lists_and_lengths(tree), 1.0)
        g.accept()
    ref.likelihood()
    tree.accept()
    ref.accept()
    L = tree.num_leaves
    seen_far = False
    for _ in range(12):
        for _ in range(4):  # four height changes in one proposal
            v = int(rng.integers(L, tree.num_nodes))
            lo = max(tree.heights[x] for x in tree.children_of(v))
            p = tree.parent_of(v)
            hi = tree.heights[p] if p is not None else lo + 2.0
            tree.set_height(v, lo + (hi - lo) * rng.uniform(0.05, 0.95))
        internals, children, lengths = lists_and_lengths(tree)
        if len(internals) > 48:
            tree.reject(); ref.reject()  # noqa: E702
            continue
        pos = {int(v): i for i, v in enumerate(internals)}
        for i, (l, r) in enumerate(children):
            for ch in (int(l), int(r)):
                if ch in pos and pos[ch] < i - 2:
                    seen_far = True
        want = ref.likelihood()
        fused.propose_lengths(internals, children, lengths, 1.0)
        two.propose_lengths(internals, children, lengths, 1.0)
        a, b = fused.log_likelihood(), two.log_likelihood()
        assert a == pytest.approx(want, rel=F32_TOL)
        assert a == pytest.approx(b, rel=1e-12, abs=0.0)
        np.testing.assert_array_equal(fused.site_log_likelihoods(),
                                      two.site_log_likelihoods())
        tree.accept(); ref.accept()  # noqa: E702
        fused.accept(); two.accept()  # noqa: E702
    assert seen_far
    fused.close()
    two.close()


def test_full_size_incremental_equals_fresh_full_recompute(rng):
    """256 taxa x 20,000 sites: fused incremental evaluations keep partials
    identical to a fresh whole-tree evaluation (run-synchronous kernel)."""
    c = dna_case(256, 20000, seed=4, model="gtr", root_height=1.0, alpha=0.5,
                 num_categories=4, pi_conc=5.0)
    fused, _two = make_pair(c, 4, 0.5)
    _two.close()
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    tree.mark_all_edges_updated()
    fused.propose_lengths(*lists_and_lengths(tree), 1.0)
    fused.accept()
    tree.accept()
    for _ in range(6):
        random_move(tree, rng)
        inc = lists_and_lengths(tree)
        if len(inc[0]) > 48:
            tree.reject()
            continue
        fused.propose_lengths(*inc, 1.0)
        d = fused.log_likelihood()
        fresh = make_gpu(c.leaves, c.weights, 4, "f32")
        fresh.set_reversible(c.rates, c.pi)
        fresh.set_gamma(0.5)
        fresh.propose_lengths(*lists_and_lengths(full(np.array(tree.parents),
                                                      np.array(tree.heights))), 1.0)
        assert d == pytest.approx(fresh.log_likelihood(), rel=1e-12, abs=0.0)
        np.testing.assert_array_equal(fused.site_log_likelihoods(),
                                      fresh.site_log_likelihoods())
        fresh.close()
        tree.accept()
        fused.accept()
    fused.close()

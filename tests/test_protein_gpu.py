"""20-state (protein) GPU path against the generic-S oracle.

Tolerances (relative, on the log-likelihood): FP64 plain form 1e-10, FP32
chosen form 1e-6.  Dirty-path evaluations must equal a fresh whole-tree
evaluation bit for bit in the FP64 form.
"""

import numpy as np
import pytest

from oracle import generic as G
from oracle import oracle as O
from tests.cases import protein_case
from tests.test_gpu_parity import F32_TOL, F64_TOL, lists_and_lengths
from tests.test_oracle import random_move

pytestmark = pytest.mark.gpu


def make20(c, precision, K, scale_ln=30):
    from aspartik_gb300.calculator import Calculator

    g = Calculator.GB300(0, precision).with_scale(scale_ln).make20(
        c.leaves, c.leaves.shape[1], num_categories=K)
    g.set_weights(c.weights)
    return g


def whole(tree):
    tree.mark_all_edges_updated()
    return lists_and_lengths(tree)


@pytest.mark.parametrize("precision,tol", [("f64", F64_TOL), ("f32", F32_TOL)])
@pytest.mark.parametrize("K,alpha", [(1, None), (4, 1.0), (3, 0.4)])
def test_whole_tree_matches_generic_oracle(precision, tol, K, alpha):
    c = protein_case(32, 600, seed=30 + K, alpha=alpha, num_categories=K, gaps=0.03)
    model = O.reversible(c.rates, c.pi)
    cats = O.gamma_categories(alpha, K) if alpha else None
    want_site = G.site_log_likelihoods(c.leaves, c.tree.parents, c.tree.heights, model, cats)
    want = float(want_site @ c.weights.astype(np.float64))
    g = make20(c, precision, K)
    g.set_reversible(c.rates, c.pi)
    if K > 1:
        g.set_gamma(alpha)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    g.propose_lengths(*whole(tree), 1.0)
    assert g.log_likelihood() == pytest.approx(want, rel=tol)
    np.testing.assert_allclose(g.site_log_likelihoods(), want_site,
                               rtol=1e-9 if precision == "f64" else 2e-5)
    g.close()


def test_calculator_level_matrices_match_oracle():
    """propose() with explicit matrices (calculator level, one category)."""
    c = protein_case(16, 300, seed=41, alpha=None, num_categories=1)
    model = O.reversible(c.rates, c.pi)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    internals, children, lengths = whole(tree)
    mats = np.array([[model.transition(d) for d in pair] for pair in lengths])
    want = G.prune(c.leaves, internals, children, mats, c.pi)
    for precision, rtol in (("f64", 1e-10), ("f32", 1e-5)):
        g = make20(c, precision, 1)
        g.propose(internals, children, mats.reshape(len(internals), 2, 1, 20, 20), c.pi)
        np.testing.assert_allclose(g.likelihoods(), want, rtol=rtol)
        g.close()


def test_dirty_paths_equal_full_recompute(rng):
    c = protein_case(48, 800, seed=43, alpha=1.0, num_categories=4, gaps=0.02)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    g64, g32 = make20(c, "f64", 4), make20(c, "f32", 4)
    for g in (g64, g32):
        g.set_reversible(c.rates, c.pi)
        g.set_gamma(1.0)
        g.propose_lengths(*whole(tree), 1.0)
        g.accept()
    tree.accept()
    for step in range(12):
        random_move(tree, rng)
        inc = lists_and_lengths(tree)
        for g in (g64, g32):
            g.propose_lengths(*inc, 1.0)
        d64, d32 = g64.log_likelihood(), g32.log_likelihood()
        fresh = make20(c, "f64", 4)
        fresh.set_reversible(c.rates, c.pi)
        fresh.set_gamma(1.0)
        fresh.propose_lengths(*whole(O.DatedTree(np.array(tree.parents),
                                                 np.array(tree.heights))), 1.0)
        assert d64 == fresh.log_likelihood(), step  # bit-identical
        assert d32 == pytest.approx(d64, rel=F32_TOL), step
        fresh.close()
        if rng.random() < 0.5:
            tree.accept()
            g64.accept()
            g32.accept()
        else:
            tree.reject()
            g64.reject()
            g32.reject()
    g64.close()
    g32.close()


def test_protein_workload_forms_agree():
    """128 taxa x 5,000 sites, 20 states, Gamma4 alpha = 1: the FP32 chosen
    form within 1e-6 of the FP64 plain form."""
    c = protein_case(128, 5000, seed=4, alpha=1.0, num_categories=4)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    lists = whole(tree)
    out = {}
    for precision in ("f64", "f32"):
        g = make20(c, precision, 4)
        g.set_reversible(c.rates, c.pi)
        g.set_gamma(1.0)
        g.propose_lengths(*lists, 1.0)
        out[precision] = g.log_likelihood()
        g.close()
    assert np.isfinite(out["f64"])
    assert out["f32"] == pytest.approx(out["f64"], rel=F32_TOL)


def make20_cuda_cores(c, K):
    """FP32 calculator that walks on the CUDA cores instead of the tensor
    cores (B3G_TC20=0 at construction)."""
    import os

    old = os.environ.get("B3G_TC20")
    os.environ["B3G_TC20"] = "0"
    try:
        return make20(c, "f32", K)
    finally:
        if old is None:
            os.environ.pop("B3G_TC20", None)
        else:
            os.environ["B3G_TC20"] = old


def test_tensor_core_path_matches_cuda_core_walk(rng):
    """3xTF32 MMAs (FP32 accumulation) against the FP32 CUDA-core walk and
    the FP64 form, whole tree and dirty paths."""
    c = protein_case(40, 700, seed=47, alpha=0.8, num_categories=4, gaps=0.02)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    tc, cc, g64 = make20(c, "f32", 4), make20_cuda_cores(c, 4), make20(c, "f64", 4)
    for g in (tc, cc, g64):
        g.set_reversible(c.rates, c.pi)
        g.set_gamma(0.8)
        g.propose_lengths(*whole(tree), 1.0)
        g.accept()
    tree.accept()
    for step in range(10):
        random_move(tree, rng)
        inc = lists_and_lengths(tree)
        for g in (tc, cc, g64):
            g.propose_lengths(*inc, 1.0)
        a, b, ref = tc.log_likelihood(), cc.log_likelihood(), g64.log_likelihood()
        assert a == pytest.approx(ref, rel=F32_TOL), step
        assert a == pytest.approx(b, rel=F32_TOL), step
        np.testing.assert_allclose(tc.site_log_likelihoods(), g64.site_log_likelihoods(),
                                   rtol=2e-5)
        tree.accept()
        for g in (tc, cc, g64):
            g.accept()
    for g in (tc, cc, g64):
        g.close()


def make20_env(c, K, **env):
    """FP32 calculator built with the given environment switches."""
    import os

    old = {k: os.environ.get(k) for k in env}
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        return make20(c, "f32", K)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


@pytest.mark.parametrize("taxa,sites,K", [(40, 700, 4), (300, 400, 2), (600, 200, 1)])
def test_tensor_core_groups_agree(rng, taxa, sites, K):
    """One and two 128-thread groups per CTA compute every entry with the
    same arithmetic and only order independent entries differently, so
    their likelihoods are bit-identical, whole tree and dirty paths; both
    meet the FP32 bar against the FP64 form.  The 600-taxon list does not
    fit shared memory beside two groups' operand areas and is read from
    global memory."""
    c = protein_case(taxa, sites, seed=53 + taxa, alpha=0.7 if K > 1 else None,
                     num_categories=K, gaps=0.02)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    g1, g2 = make20_env(c, K, B3G_TC20_GROUPS=1), make20_env(c, K, B3G_TC20_GROUPS=2)
    g64 = make20(c, "f64", K)
    for g in (g1, g2, g64):
        g.set_reversible(c.rates, c.pi)
        if K > 1:
            g.set_gamma(0.7)
        g.propose_lengths(*whole(tree), 1.0)
    a, b, ref = g1.log_likelihood(), g2.log_likelihood(), g64.log_likelihood()
    assert a == b
    assert a == pytest.approx(ref, rel=F32_TOL)
    np.testing.assert_array_equal(g1.site_log_likelihoods(), g2.site_log_likelihoods())
    for g in (g1, g2, g64):
        g.accept()
    tree.accept()
    for step in range(6):
        random_move(tree, rng)
        inc = lists_and_lengths(tree)
        for g in (g1, g2, g64):
            g.propose_lengths(*inc, 1.0)
        a, b, ref = g1.log_likelihood(), g2.log_likelihood(), g64.log_likelihood()
        assert a == b, step
        assert a == pytest.approx(ref, rel=F32_TOL), step
        tree.accept()
        for g in (g1, g2, g64):
            g.accept()
    for g in (g1, g2, g64):
        g.close()


@pytest.mark.parametrize("groups", [1, 2])
def test_tensor_core_single_entry_lists_and_eight_categories(groups):
    """Root-only dirty lists (one entry: one run, the second group idle),
    then lists of the root's internal child and the root, on the tensor
    cores with eight Gamma categories and with one pattern (a single
    tile, 127 padded rows), each against the FP64 form."""
    for taxa, sites, K in ((24, 400, 8), (12, 1, 2)):
        c = protein_case(taxa, sites, seed=61 + K, alpha=0.6, num_categories=K)
        tree = O.DatedTree(c.tree.parents, c.tree.heights)
        tc = make20_env(c, K, B3G_TC20_GROUPS=groups)
        g64 = make20(c, "f64", K)
        for g in (tc, g64):
            g.set_reversible(c.rates, c.pi)
            g.set_gamma(0.6)
            g.propose_lengths(*whole(tree), 1.0)
            g.accept()
        tree.accept()
        root = tree.root()
        l, r = tree.children_of(root)
        top = max(tree.heights[l], tree.heights[r])
        for step, h in enumerate((top + 0.3, top + 0.05, top + 1.1)):
            tree.set_height(root, h)
            inc = lists_and_lengths(tree)
            assert len(inc[0]) == 1
            for g in (tc, g64):
                g.propose_lengths(*inc, 1.0)
            assert tc.log_likelihood() == pytest.approx(g64.log_likelihood(), rel=F32_TOL), step
            tree.accept()
            for g in (tc, g64):
                g.accept()
        inner = next((v for v in (l, r) if v >= tree.num_leaves), None)
        if inner is not None:
            a, b = tree.children_of(inner)
            lo, hi = max(tree.heights[a], tree.heights[b]), tree.heights[root]
            tree.set_height(inner, lo + 0.5 * (hi - lo))
            inc = lists_and_lengths(tree)
            assert len(inc[0]) == 2
            for g in (tc, g64):
                g.propose_lengths(*inc, 1.0)
            assert tc.log_likelihood() == pytest.approx(g64.log_likelihood(), rel=F32_TOL)
        tc.close()
        g64.close()


@pytest.mark.parametrize("groups", [1, 2])
def test_tensor_core_clusters_agree(rng, groups):
    """A work item (pattern tile, category) spread over a thread-block
    cluster of 2, 3 or 8 CTAs walks every run's independent entries on more
    groups (a cluster barrier between runs, partials passed through global
    memory) with the same per-entry arithmetic: the likelihoods equal one
    CTA per item bit for bit, whole tree and dirty paths, and meet the FP32
    bar against the FP64 form."""
    c = protein_case(48, 600, seed=71, alpha=0.6, num_categories=4, gaps=0.02)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    calcs = {k: make20_env(c, 4, B3G_TC20_GROUPS=groups, B3G_TC20_CLUSTER=k)
             for k in (1, 2, 3, 8)}
    g64 = make20(c, "f64", 4)
    every = list(calcs.values()) + [g64]
    for g in every:
        g.set_reversible(c.rates, c.pi)
        g.set_gamma(0.6)
        g.propose_lengths(*whole(tree), 1.0)
    ref = g64.log_likelihood()
    base = calcs[1].log_likelihood()
    assert base == pytest.approx(ref, rel=F32_TOL)
    for k, g in calcs.items():
        assert g.log_likelihood() == base, k
        np.testing.assert_array_equal(g.site_log_likelihoods(),
                                      calcs[1].site_log_likelihoods())
    for g in every:
        g.accept()
    tree.accept()
    for step in range(5):
        random_move(tree, rng)
        inc = lists_and_lengths(tree)
        for g in every:
            g.propose_lengths(*inc, 1.0)
        base = calcs[1].log_likelihood()
        assert base == pytest.approx(g64.log_likelihood(), rel=F32_TOL), step
        for k, g in calcs.items():
            assert g.log_likelihood() == base, (step, k)
        tree.accept()
        for g in every:
            g.accept()
    for g in every:
        g.close()

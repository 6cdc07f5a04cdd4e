"""The CPU oracle against independent ground truth (CPU only).

The reference ships no golden likelihood for this path (its trace tests read
an absent data submodule), so the oracle is pinned against brute-force
enumeration (tests/golden), closed forms, scipy's expm and gammaincinv, and
against itself through invariances the reference's own tests use
(scale_ln in {3, 30, 300}, python/tests/b3/likelihoods_comp.py:10-33)."""

import os

import numpy as np
import pytest
from scipy.linalg import expm
from scipy.special import gammaincinv

from aspartik_gb300 import sim
from oracle import brute
from oracle import oracle as O
from tests.cases import dna_case

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "small_trees.npz")


def golden_cases():
    g = np.load(GOLDEN)
    names = sorted({k.split("/")[0] for k in g.files})
    return g, names


def model_for(pi, rates):
    return O.gtr(rates, pi)


@pytest.mark.parametrize("name", golden_cases()[1])
def test_oracle_matches_golden(name):
    g, _ = golden_cases()
    f = lambda k: g[f"{name}/{k}"]  # noqa: E731
    tree = O.DatedTree(f("parents"), f("heights"))
    model = model_for(f("pi"), f("rates"))
    K = int(f("categories"))
    if K == 1:
        lik = O.DnaLikelihood(f("leaves"), f("weights"), tree, model)
    else:
        lik = O.GammaLikelihood(f("leaves"), f("weights"), tree, model, K, float(f("alpha")))
    assert lik.cache == pytest.approx(float(f("lnl")), rel=1e-12)


def test_golden_regenerates_identically():
    """The committed fixtures are what make_golden.py produces."""
    import subprocess
    import sys
    import tempfile

    g, names = golden_cases()
    with tempfile.TemporaryDirectory() as d:
        script = os.path.join(os.path.dirname(__file__), "golden", "make_golden.py")
        src = open(script).read().replace(
            'OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_trees.npz")',
            f'OUT = {os.path.join(d, "x.npz")!r}')
        tmp = os.path.join(d, "gen.py")
        open(tmp, "w").write(src.replace(
            "ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))",
            f"ROOT = {os.path.dirname(os.path.dirname(os.path.abspath(__file__)))!r}"))
        subprocess.run([sys.executable, tmp], check=True, capture_output=True)
        h = np.load(os.path.join(d, "x.npz"))
        for k in g.files:
            np.testing.assert_array_equal(g[k], h[k])


def test_jc_k80_hky_closed_forms_agree_with_expm(rng):
    for d in [1e-9, 1e-3, 0.1, 1.0, 5.0, 19.0]:
        Qjc = sim.reversible_q(np.ones(6), np.full(4, 0.25))
        np.testing.assert_allclose(O.JC().transition(d), expm(Qjc * d), rtol=0, atol=1e-14)
        kappa = 3.0
        Qk = sim.reversible_q(sim.hky_rates(kappa), np.full(4, 0.25))
        np.testing.assert_allclose(O.K80(kappa).transition(d), expm(Qk * d), rtol=0, atol=1e-14)
        pi = sim.dirichlet([10] * 4, rng)
        m = O.hky(2.0, pi)
        Qh = sim.reversible_q(sim.hky_rates(2.0), pi)
        np.testing.assert_allclose(m.Q.reshape(4, 4), Qh, rtol=1e-13, atol=1e-15)
        if d >= 1e-10:
            np.testing.assert_allclose(m.transition(d), expm(Qh * d), rtol=0, atol=1e-13)


def test_hky_shortcuts():
    pi = np.array([0.1, 0.2, 0.3, 0.4])
    m = O.hky(2.0, pi)
    np.testing.assert_array_equal(m.transition(25.0), np.tile(pi, (4, 1)))
    small = m.transition(1e-12)
    np.testing.assert_array_equal(np.diag(small), np.ones(4))
    off = small - np.diag(np.diag(small))
    np.testing.assert_allclose(off, (m.Q.reshape(4, 4) * 1e-12) * (1 - np.eye(4)))


def test_gtr_eigen_agrees_with_expm(rng):
    for _ in range(5):
        pi = sim.dirichlet([5] * 4, rng)
        rates = rng.gamma(2.0, 1.0, size=6)
        m = O.gtr(rates, pi)
        Q = sim.reversible_q(rates, pi)
        np.testing.assert_allclose(m.Q.reshape(4, 4), Q, rtol=1e-12, atol=1e-15)
        for d in [1e-6, 0.05, 0.7, 4.0]:
            np.testing.assert_allclose(m.transition(d), expm(Q * d), rtol=0, atol=1e-13)


def test_20_state_eigen_agrees_with_expm(rng):
    pi = sim.dirichlet([1.0] * 20, rng)
    rates = rng.lognormal(0.0, 1.0, size=190)
    m = O.reversible(rates, pi)
    Q = sim.reversible_q(rates, pi)
    for d in [0.01, 0.3, 2.0]:
        np.testing.assert_allclose(m.transition(d), expm(Q * d), rtol=0, atol=1e-12)
    # JC-20 closed form: P_ii = 1/20 + 19/20 exp(-20 t / 19)
    mj = O.reversible(np.ones(190), np.full(20, 0.05))
    for t in [0.1, 1.0]:
        P = mj.transition(t)
        np.testing.assert_allclose(np.diag(P), 0.05 + 0.95 * np.exp(-20 * t / 19), rtol=1e-13)


@pytest.mark.parametrize("alpha", [0.05, 0.2, 0.5, 1.0, 2.0, 10.0, 200.0])
@pytest.mark.parametrize("k", [1, 2, 4, 8])
def test_gamma_categories_match_scipy(alpha, k):
    ours = O.gamma_categories(alpha, k)
    q = gammaincinv(alpha, (2 * np.arange(k) + 1) / (2 * k))
    np.testing.assert_allclose(ours, q / q.mean(), rtol=1e-12)


@pytest.mark.parametrize("scale_ln", [3, 30, 300])
def test_scale_invariance(scale_ln):
    """The rescaling threshold changes no likelihood (the idea of
    python/tests/b3/likelihoods_comp.py:10-33)."""
    c = dna_case(64, 400, seed=7, model="gtr", root_height=2.0)
    ref = O.DnaLikelihood(c.leaves, c.weights, O.DatedTree(c.tree.parents, c.tree.heights),
                          O.gtr(c.rates, c.pi), scale_ln=30).cache
    got = O.DnaLikelihood(c.leaves, c.weights, O.DatedTree(c.tree.parents, c.tree.heights),
                          O.gtr(c.rates, c.pi), scale_ln=scale_ln).cache
    assert got == pytest.approx(ref, rel=1e-12)


def test_deduplication_preserves_likelihood():
    c = dna_case(8, 300, seed=11, gaps=0.05)
    leaves, w, s2p = O.deduplicate(c.msa)
    assert leaves.shape[1] < c.msa.shape[1]
    assert w.sum() == c.msa.shape[1]
    raw = c.msa.copy()
    raw[raw == 0] = 0x0F
    tree = lambda: O.DatedTree(c.tree.parents, c.tree.heights)  # noqa: E731
    m = O.hky(2.0, c.pi)
    a = O.DnaLikelihood(leaves, w, tree(), m).cache
    b = O.DnaLikelihood(raw, np.ones(raw.shape[1], np.uint32), tree(), m).cache
    assert a == pytest.approx(b, rel=1e-12)
    # numpy and C deduplication agree exactly
    l2, w2, s2 = sim.deduplicate(c.msa)
    np.testing.assert_array_equal(leaves, l2)
    np.testing.assert_array_equal(w, w2)
    np.testing.assert_array_equal(s2p, s2)


def random_move(tree: O.DatedTree, rng):
    """A height change of a random internal within its bounds, or an
    exchange of two nodes (narrow exchange), as b3's operators do."""
    L = tree.num_leaves
    if rng.random() < 0.6:
        v = int(rng.integers(L, tree.num_nodes))
        l, r = tree.children_of(v)
        lo = max(tree.heights[l], tree.heights[r])
        p = tree.parent_of(v)
        hi = tree.heights[p] if p is not None else lo + 2.0
        tree.set_height(v, lo + (hi - lo) * rng.uniform(0.05, 0.95))
    else:
        # narrow exchange: grandparent g, parent p (child of g), uncle u,
        # nephew n (child of p) with height(n) < height(g); swap n and u
        cands = []
        for g in range(L, tree.num_nodes):
            for p in tree.children_of(g):
                if p >= L:
                    u = [x for x in tree.children_of(g) if x != p][0]
                    for n in tree.children_of(p):
                        if tree.heights[u] < tree.heights[p] and tree.heights[n] < tree.heights[g]:
                            cands.append((g, p, u, n))
        if not cands:
            return
        g, p, u, n = cands[int(rng.integers(len(cands)))]
        tree.replace_child(g, u, n)
        tree.replace_child(p, n, u)


def test_dirty_path_equals_full_recompute(rng):
    """Random proposals with accept/reject: the incremental likelihood always
    equals a fresh full evaluation (hardens python/tests/b3/likelihoods.py)."""
    c = dna_case(12, 200, seed=5)
    m = O.hky(2.0, c.pi)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    lik = O.DnaLikelihood(c.leaves, c.weights, tree, m)
    for _ in range(60):
        random_move(tree, rng)
        tree.validate()
        got = lik.likelihood()
        fresh = O.DnaLikelihood(c.leaves, c.weights,
                                O.DatedTree(np.array(tree.parents), np.array(tree.heights)),
                                m).cache
        assert got == pytest.approx(fresh, rel=1e-12)
        if rng.random() < 0.5:
            tree.accept()
            lik.accept()
        else:
            tree.reject()
            lik.reject()


def test_multithreaded_oracle_is_thread_count_invariant():
    c = dna_case(16, 3000, seed=9)
    vals = []
    for t in (1, 3, 8):
        calc = O.Cpu4Calculator(c.leaves, c.weights.size, 30, t)
        assert calc.num_threads() == t
        tree = O.DatedTree(c.tree.parents, c.tree.heights)
        tree.mark_all_edges_updated()
        internals, children = tree.partials_lists()
        m = O.hky(2.0, c.pi)
        mats = np.stack([m.transition(tree.edge_length(e)) for e in children.reshape(-1)])
        calc.propose(internals, children, mats, c.pi)
        vals.append(calc.likelihoods())
    np.testing.assert_array_equal(vals[0], vals[1])
    np.testing.assert_array_equal(vals[0], vals[2])


def test_brute_force_small_cases_agree_with_oracle(rng):
    for seed in range(3):
        c = dna_case(int(rng.integers(2, 7)), 30, seed=100 + seed, model="gtr", gaps=0.1)
        Q = sim.reversible_q(c.rates, c.pi)
        site = brute.site_log_likelihoods(c.tree.parents, c.tree.heights, c.leaves, Q, c.pi)
        lik = O.DnaLikelihood(c.leaves, c.weights, O.DatedTree(c.tree.parents, c.tree.heights),
                              O.gtr(c.rates, c.pi))
        assert lik.cache == pytest.approx(float((site * c.weights).sum()), rel=1e-12)

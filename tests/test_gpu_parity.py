"""GPU parity: the sm_103a path through the C ABI against the CPU oracle and
the brute-force golden vectors.

Tolerances (relative, on the log-likelihood):
  FP64 plain form   1e-10  (the bar of the drop-in)
  FP32 chosen form  1e-6
Integer bookkeeping (dirty lists, selectors, rescale counts) must give
results identical to a full recompute.
"""

import os

import numpy as np
import pytest

from aspartik_gb300 import sim
from oracle import oracle as O
from tests.cases import dna_case

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10
F32_TOL = 1e-6
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "small_trees.npz")


def calc_cls():
    from aspartik_gb300.calculator import Calculator

    return Calculator


def lists_and_lengths(tree: O.DatedTree):
    internals, children = tree.partials_lists()
    lengths = np.array([[tree.edge_length(int(a)), tree.edge_length(int(b))]
                        for a, b in children]).reshape(-1, 2)
    return internals, children, lengths


def full(tree_parents, tree_heights):
    t = O.DatedTree(tree_parents, tree_heights)
    t.mark_all_edges_updated()
    return t


def make_gpu(leaves, weights, K=1, precision="f64", scale_ln=30):
    c = calc_cls().GB300(0, precision).with_scale(scale_ln).make4(
        leaves, leaves.shape[1], num_categories=K)
    c.set_weights(weights)
    return c


# --------------------------------------------------------------------------
# golden vectors (brute force)

def golden_names():
    g = np.load(GOLDEN)
    return sorted({k.split("/")[0] for k in g.files})


@pytest.mark.parametrize("precision,tol", [("f64", F64_TOL), ("f32", F32_TOL)])
@pytest.mark.parametrize("name", golden_names())
def test_golden_likelihood_level(name, precision, tol):
    g = np.load(GOLDEN)
    f = lambda k: g[f"{name}/{k}"]  # noqa: E731
    K = int(f("categories"))
    calc = make_gpu(f("leaves"), f("weights"), K, precision)
    calc.set_reversible(f("rates"), f("pi"))
    calc.set_category_rates(f("cat_rates"))
    internals, children, lengths = lists_and_lengths(full(f("parents"), f("heights")))
    calc.propose_lengths(internals, children, lengths, 1.0)
    assert calc.log_likelihood() == pytest.approx(float(f("lnl")), rel=tol)
    np.testing.assert_allclose(calc.site_log_likelihoods(), f("site_lnl"), rtol=tol * 10,
                               atol=tol)


@pytest.mark.parametrize("name", golden_names())
def test_golden_calculator_level(name):
    """The trait-level drop-in: per-pattern likelihoods from the reference's
    inputs (dirty list, gathered matrices, frequencies)."""
    g = np.load(GOLDEN)
    f = lambda k: g[f"{name}/{k}"]  # noqa: E731
    if int(f("categories")) != 1:
        pytest.skip("calculator level is one category per calculator")
    tree = full(f("parents"), f("heights"))
    model = O.gtr(f("rates"), f("pi"))
    internals, children = tree.partials_lists()
    mats = np.stack([model.transition(tree.edge_length(int(e))) for e in children.reshape(-1)])
    calc = make_gpu(f("leaves"), f("weights"))
    calc.propose(internals, children, mats, f("pi"))
    np.testing.assert_allclose(calc.likelihoods(), f("site_lnl"), rtol=1e-12, atol=1e-12)


# --------------------------------------------------------------------------
# oracle parity, calculator level

@pytest.mark.parametrize("L,N,scale_ln", [(2, 50, 30), (3, 10, 30), (16, 1000, 30),
                                          (64, 700, 3), (64, 700, 300), (40, 129, 30)])
def test_calculator_level_matches_cpu4(L, N, scale_ln):
    c = dna_case(L, N, seed=L + N, model="gtr", root_height=2.5, gaps=0.05)
    tree = full(c.tree.parents, c.tree.heights)
    model = O.gtr(c.rates, c.pi)
    internals, children = tree.partials_lists()
    mats = np.stack([model.transition(tree.edge_length(int(e))) for e in children.reshape(-1)])
    cpu = O.Cpu4Calculator(c.leaves, c.weights.size, scale_ln)
    cpu.propose(internals, children, mats, c.pi)
    gpu = make_gpu(c.leaves, c.weights, scale_ln=scale_ln)
    gpu.propose(internals, children, mats, c.pi)
    np.testing.assert_allclose(gpu.likelihoods(), cpu.likelihoods(), rtol=1e-12, atol=1e-11)


def test_calculator_level_random_sequences(rng):
    """propose / accept / reject in random order against the oracle, with the
    dirty lists the reference's tree produces."""
    from tests.test_oracle import random_move

    c = dna_case(20, 300, seed=21)
    model = O.hky(2.0, c.pi)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    tree.mark_all_edges_updated()
    cpu = O.Cpu4Calculator(c.leaves, c.weights.size)
    gpu = make_gpu(c.leaves, c.weights)
    for step in range(80):
        if step:
            random_move(tree, rng)
        internals, children = tree.partials_lists()
        mats = np.stack([model.transition(tree.edge_length(int(e)))
                         for e in children.reshape(-1)])
        cpu.propose(internals, children, mats, c.pi)
        gpu.propose(internals, children, mats, c.pi)
        np.testing.assert_allclose(gpu.likelihoods(), cpu.likelihoods(), rtol=1e-12, atol=1e-11)
        if rng.random() < 0.5:
            tree.accept(); cpu.accept(); gpu.accept()  # noqa: E702
        else:
            tree.reject(); cpu.reject(); gpu.reject()  # noqa: E702


# --------------------------------------------------------------------------
# oracle parity, likelihood level (DnaLikelihood / GammaLikelihood)

@pytest.mark.parametrize("precision,tol", [("f64", F64_TOL), ("f32", F32_TOL)])
@pytest.mark.parametrize("K,alpha", [(1, None), (4, 0.5), (3, 1.3), (8, 0.2)])
def test_gamma_likelihood_matches_oracle(precision, tol, K, alpha):
    c = dna_case(64, 2000, seed=64 + K, model="gtr", root_height=1.0,
                 alpha=alpha, num_categories=K, gaps=0.02)
    model = O.gtr(c.rates, c.pi)
    t = O.DatedTree(c.tree.parents, c.tree.heights)
    if K == 1:
        ref = O.DnaLikelihood(c.leaves, c.weights, t, model).cache
    else:
        ref = O.GammaLikelihood(c.leaves, c.weights, t, model, K, alpha).cache
    gpu = make_gpu(c.leaves, c.weights, K, precision)
    gpu.set_reversible(c.rates, c.pi)
    if K > 1:
        gpu.set_gamma(alpha)
    internals, children, lengths = lists_and_lengths(full(c.tree.parents, c.tree.heights))
    gpu.propose_lengths(internals, children, lengths, 1.0)
    assert gpu.log_likelihood() == pytest.approx(ref, rel=tol)


def test_hky_analytic_eigensystem_with_shortcuts():
    """The host-provided eigensystem path with the d > 20 and d < 1e-10
    shortcuts of HKY::write_transition (substitution.rs:403-420)."""
    c = dna_case(10, 200, seed=3, root_height=1.0)
    parents, heights = c.tree.parents.copy(), c.tree.heights.copy()
    heights[0] = heights[parents[0]] - 1e-12   # a branch shorter than 1e-10
    heights[1] = -30.0                          # a branch longer than 20
    m = O.hky(2.0, c.pi)
    ref = O.DnaLikelihood(c.leaves, c.weights, O.DatedTree(parents, heights), m).cache
    gpu = make_gpu(c.leaves, c.weights)
    gpu.set_eigen(m.V, m.Vinv, m.lam, m.Q, m.pi, shortcuts=True)
    internals, children, lengths = lists_and_lengths(full(parents, heights))
    gpu.propose_lengths(internals, children, lengths, 1.0)
    assert gpu.log_likelihood() == pytest.approx(ref, rel=F64_TOL)


def test_mcmc_like_sequence_matches_oracle(rng):
    """Moves, model changes, accept and reject: after every step the GPU
    likelihood equals the oracle's, in both forms."""
    from tests.test_oracle import random_move

    c = dna_case(32, 800, seed=33, model="gtr", alpha=0.5, num_categories=4)
    rates, pi, alpha = c.rates.copy(), c.pi.copy(), 0.5
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    ref = O.GammaLikelihood(c.leaves, c.weights, tree, O.gtr(rates, pi), 4, alpha)
    gpus = {p: make_gpu(c.leaves, c.weights, 4, p) for p in ("f64", "f32")}
    for g in gpus.values():
        g.set_reversible(rates, pi)
        g.set_gamma(alpha)
        g.propose_lengths(*lists_and_lengths(full(c.tree.parents, c.tree.heights)), 1.0)
        g.accept()
    for step in range(40):
        kind = rng.random()
        new_rates, new_alpha = rates, alpha
        if kind < 0.15:
            new_rates = rates * np.exp(rng.normal(0, 0.1, 6))
            ref.set_model(O.gtr(new_rates, pi))
        elif kind < 0.25:
            new_alpha = alpha * float(np.exp(rng.normal(0, 0.2)))
            ref.set_alpha(new_alpha)
        else:
            random_move(tree, rng)
        internals, children, lengths = lists_and_lengths(tree)
        want = ref.likelihood()
        for p, g in gpus.items():
            if new_rates is not rates:
                g.set_reversible(new_rates, pi)
            if new_alpha != alpha:
                g.set_gamma(new_alpha)
            g.propose_lengths(internals, children, lengths, 1.0)
            got = g.log_likelihood()
            assert got == pytest.approx(want, rel=F64_TOL if p == "f64" else F32_TOL), (step, p)
        if rng.random() < 0.5:
            tree.accept(); ref.accept()  # noqa: E702
            for g in gpus.values():
                g.accept()
            rates, alpha = new_rates, new_alpha
        else:
            tree.reject(); ref.reject()  # noqa: E702
            for g in gpus.values():
                g.reject()
                if new_rates is not rates:
                    g.set_reversible(rates, pi)
                if new_alpha != alpha:
                    g.set_gamma(alpha)
            if new_rates is not rates:
                ref.model = O.gtr(rates, pi)
            if new_alpha != alpha:
                ref.alpha = alpha
                ref.categories = O.gamma_categories(alpha, 4)


# --------------------------------------------------------------------------
# edge cases

def test_single_pattern_and_all_unknown_columns():
    c = dna_case(6, 1, seed=2)
    gpu = make_gpu(c.leaves, c.weights)
    gpu.set_reversible(np.ones(6), np.full(4, 0.25))
    gpu.propose_lengths(*lists_and_lengths(full(c.tree.parents, c.tree.heights)), 1.0)
    ref = O.DnaLikelihood(c.leaves, c.weights, O.DatedTree(c.tree.parents, c.tree.heights),
                          O.gtr(np.ones(6), np.full(4, 0.25))).cache
    assert gpu.log_likelihood() == pytest.approx(ref, rel=F64_TOL)
    # an all-gap column has likelihood 1 (log 0) under every model
    leaves = np.full((6, 3), 0x0F, dtype=np.uint8)
    gpu = make_gpu(leaves, np.array([1, 2, 3], np.uint32))
    gpu.set_reversible(np.ones(6), np.full(4, 0.25))
    gpu.propose_lengths(*lists_and_lengths(full(c.tree.parents, c.tree.heights)), 1.0)
    assert abs(gpu.log_likelihood()) < 1e-12


def test_zero_length_branch_gives_impossible_pattern():
    """Two different bases on a cherry with zero-length branches have
    likelihood 0: lnL = -inf in both forms, as in the oracle."""
    parents = np.array([2, 2, 0xFFFFFFFF], dtype=np.uint32)
    heights = np.array([0.0, 0.0, 0.0])
    leaves = np.array([[1], [2]], dtype=np.uint8)
    ref = O.DnaLikelihood(leaves, np.ones(1, np.uint32), O.DatedTree(parents, heights),
                          O.hky(2.0, np.full(4, 0.25))).cache
    assert ref == -np.inf
    for p in ("f64", "f32"):
        gpu = make_gpu(leaves, np.ones(1, np.uint32), 1, p)
        m = O.hky(2.0, np.full(4, 0.25))
        gpu.set_eigen(m.V, m.Vinv, m.lam, m.Q, m.pi)
        gpu.propose_lengths(*lists_and_lengths(full(parents, heights)), 1.0)
        assert gpu.log_likelihood() == -np.inf


def test_invalid_inputs_fail_cleanly_and_leave_state_intact():
    from aspartik_gb300._native import (B3G_ERR_INVALID_ARGUMENT, B3G_ERR_NUMERIC,
                                        B3G_ERR_STATE, B3GError)

    c = dna_case(8, 100, seed=8)
    gpu = make_gpu(c.leaves, c.weights)
    internals, children, lengths = lists_and_lengths(full(c.tree.parents, c.tree.heights))
    with pytest.raises(B3GError) as e:
        gpu.propose_lengths(internals, children, lengths)
    assert e.value.status == B3G_ERR_STATE
    with pytest.raises(B3GError) as e:
        gpu.likelihoods()
    assert e.value.status == B3G_ERR_STATE
    gpu.set_reversible(np.ones(6), c.pi)
    bad = [
        (internals[::-1].copy(), children[::-1].copy(), lengths),   # parents first
        (np.r_[internals[:-1], 0].astype(np.uint32), children, lengths),  # a leaf listed
        (np.r_[internals[:-1], 99].astype(np.uint32), children, lengths),  # out of range
        (np.r_[internals[:1], internals[:1]].astype(np.uint32), children[:2], lengths[:2]),
    ]
    for ints, ch, ln in bad:
        with pytest.raises(B3GError) as e:
            gpu.propose_lengths(ints, ch, ln)
        assert e.value.status == B3G_ERR_INVALID_ARGUMENT
    nan_len = lengths.copy()
    nan_len[0, 0] = np.nan
    with pytest.raises(B3GError) as e:
        gpu.propose_lengths(internals, children, nan_len)
    assert e.value.status == B3G_ERR_NUMERIC
    with pytest.raises(B3GError) as e:
        gpu.set_reversible(np.ones(6), np.array([0.5, 0.5, 0.0, 0.0]))
    assert e.value.status == B3G_ERR_NUMERIC
    # the failed calls changed nothing: a valid call still matches the oracle
    gpu.set_reversible(np.ones(6), c.pi)
    gpu.propose_lengths(internals, children, lengths)
    ref = O.DnaLikelihood(c.leaves, c.weights, O.DatedTree(c.tree.parents, c.tree.heights),
                          O.gtr(np.ones(6), c.pi)).cache
    assert gpu.log_likelihood() == pytest.approx(ref, rel=F64_TOL)


def test_repeated_evaluation_in_one_epoch_is_exact():
    """Proposing twice before accept/reject keeps the rescale counts exact
    (the reference's per-pattern running sum double-counts here)."""
    c = dna_case(48, 500, seed=48, root_height=4.0)
    m = O.hky(2.0, c.pi)
    gpu = make_gpu(c.leaves, c.weights, scale_ln=3)
    gpu.set_eigen(m.V, m.Vinv, m.lam, m.Q, m.pi)
    args = lists_and_lengths(full(c.tree.parents, c.tree.heights))
    gpu.propose_lengths(*args)
    a = gpu.log_likelihood()
    gpu.propose_lengths(*args)
    b = gpu.log_likelihood()
    assert a == b


# --------------------------------------------------------------------------
# full size (256 taxa, 20,000 sites, GTR + Gamma4): size-independent checks

@pytest.fixture(scope="module")
def big_case():
    return dna_case(256, 20000, seed=4, model="gtr", root_height=1.0, alpha=0.5,
                    num_categories=4, pi_conc=5.0)


def test_full_size_forms_agree_and_dirty_equals_full(big_case, rng):
    from tests.test_oracle import random_move

    c = big_case
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    tree.mark_all_edges_updated()
    g64 = make_gpu(c.leaves, c.weights, 4, "f64")
    g32 = make_gpu(c.leaves, c.weights, 4, "f32")
    for g in (g64, g32):
        g.set_reversible(c.rates, c.pi)
        g.set_gamma(0.5)
        g.propose_lengths(*lists_and_lengths(tree), 1.0)
    a64, a32 = g64.log_likelihood(), g32.log_likelihood()
    assert a32 == pytest.approx(a64, rel=F32_TOL)
    # deterministic: the same evaluation gives the same bits
    g64.propose_lengths(*lists_and_lengths(tree), 1.0)
    assert g64.log_likelihood() == a64
    for g in (g64, g32):
        g.accept()
    tree.accept()
    for _ in range(5):
        random_move(tree, rng)
        inc = lists_and_lengths(tree)
        g64.propose_lengths(*inc, 1.0)
        g32.propose_lengths(*inc, 1.0)
        d64, d32 = g64.log_likelihood(), g32.log_likelihood()
        fresh = make_gpu(c.leaves, c.weights, 4, "f64")
        fresh.set_reversible(c.rates, c.pi)
        fresh.set_gamma(0.5)
        fresh.propose_lengths(*lists_and_lengths(full(np.array(tree.parents),
                                                      np.array(tree.heights))), 1.0)
        assert d64 == fresh.log_likelihood()  # bit-identical
        assert d32 == pytest.approx(d64, rel=F32_TOL)
        fresh.close()
        tree.accept()
        g64.accept()
        g32.accept()


# --------------------------------------------------------------------------
# the configurations' sizes against the oracle: 64 taxa x 10,000 sites and
# 256 taxa x 20,000 sites, GTR + Gamma4 (exchangeabilities ~ Gamma(2, 1),
# frequencies ~ Dirichlet(5, 5, 5, 5), alpha 0.5, Yule tree of root height 1)

@pytest.mark.parametrize("L,N,seed", [(64, 10000, 2), (256, 20000, 4)])
def test_configuration_sizes_match_oracle(L, N, seed, rng):
    """Whole tree, then dirty paths with accept and reject: both forms
    against the restated GammaLikelihood (four cpu4 calculators) at every
    step, FP64 within 1e-10 and FP32 within 1e-6."""
    from tests.test_oracle import random_move

    c = dna_case(L, N, seed=seed, model="gtr", root_height=1.0, alpha=0.5,
                 num_categories=4, pi_conc=5.0)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    ref = O.GammaLikelihood(c.leaves, c.weights, tree, O.gtr(c.rates, c.pi), 4, 0.5)
    gpus = {p: make_gpu(c.leaves, c.weights, 4, p) for p in ("f64", "f32")}
    tol = {"f64": F64_TOL, "f32": F32_TOL}
    for p, g in gpus.items():
        g.set_reversible(c.rates, c.pi)
        g.set_gamma(0.5)
        g.propose_lengths(*lists_and_lengths(full(c.tree.parents, c.tree.heights)), 1.0)
        assert g.log_likelihood() == pytest.approx(ref.cache, rel=tol[p]), p
        g.accept()
    for step in range(6):
        random_move(tree, rng)
        lists = lists_and_lengths(tree)
        want = ref.likelihood()
        for p, g in gpus.items():
            g.propose_lengths(*lists, 1.0)
            assert g.log_likelihood() == pytest.approx(want, rel=tol[p]), (step, p)
        if step % 2 == 0:
            tree.accept(); ref.accept()  # noqa: E702
            for g in gpus.values():
                g.accept()
        else:
            tree.reject(); ref.reject()  # noqa: E702
            for g in gpus.values():
                g.reject()
    for g in gpus.values():
        g.close()

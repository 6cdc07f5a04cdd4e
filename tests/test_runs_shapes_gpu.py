"""The run-synchronous FP32 walk in every shape it can take: patterns per
tile, 512- or 1024-thread blocks, children kept in shared-memory slots or
read back from global memory, transition tables built per run inside the
walk or written by the separate transition kernel.  Per-pattern values are
the same bits in every shape (the per-column arithmetic does not depend on
the shape); the total is the same bits for one (tile, block) shape and
within FP64 rounding of the summation order across shapes; and the walk
agrees with the FP64 form within the FP32 tolerance.  Whole trees, dirty
lists (with the fused short-list kernel off, so that they take the run
walk too) and explicit matrices (cpu4.rs:100-118 interface)."""

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import dna_case
from tests.test_gpu_parity import F32_TOL, full, lists_and_lengths, make_gpu
from tests.test_oracle import random_move

pytestmark = pytest.mark.gpu

SHAPES = [  # (tile, block, slots, inline)
    (64, 512, 0, 0), (64, 512, 1, 0), (64, 512, 0, 1), (64, 512, 1, 1),
    (32, 512, 1, 1), (32, 1024, 1, 1), (64, 1024, 1, 1), (64, 1024, 0, 0),
    (16, 512, 1, 1), (16, 512, 0, 0), (16, 1024, 1, 1),
]


def run_sequence(c, K, alpha, shape, monkeypatch, seed):
    tile, block, slots, inline = shape
    monkeypatch.setenv("B3G_RUNS_TILE", str(tile))
    monkeypatch.setenv("B3G_RUNS_BLOCK", str(block))
    monkeypatch.setenv("B3G_RUNS_SLOTS", str(slots))
    monkeypatch.setenv("B3G_RUNS_INLINE", str(inline))
    monkeypatch.setenv("B3G_DIRECT", "0")
    rng = np.random.default_rng(seed)
    g = make_gpu(c.leaves, c.weights, K, "f32")
    g.set_reversible(c.rates, c.pi)
    if K > 1:
        g.set_gamma(alpha)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    tree.mark_all_edges_updated()
    out = []
    g.propose_lengths(*lists_and_lengths(tree), 1.0)
    out.append((g.log_likelihood(), g.site_log_likelihoods()))
    g.accept()
    tree.accept()
    for step in range(6):
        for _ in range(1 + step):  # dirty lists of growing size
            random_move(tree, rng)
        g.propose_lengths(*lists_and_lengths(tree), 0.9 + 0.05 * step)
        out.append((g.log_likelihood(), g.site_log_likelihoods()))
        if step % 2:
            g.reject()
            tree.reject()
        else:
            g.accept()
            tree.accept()
    # explicit matrices for the whole tree
    model = O.gtr(c.rates, c.pi)
    cats = O.gamma_categories(alpha, K) if K > 1 else np.ones(1)
    t2 = full(np.array(tree.parents), np.array(tree.heights))
    internals, children, lengths = lists_and_lengths(t2)
    mats = np.array([[[model.transition(d * r) for r in cats] for d in pair]
                     for pair in lengths])
    g.propose(internals, children, mats, c.pi)
    out.append((g.log_likelihood(), g.site_log_likelihoods()))
    g.reject()
    ref64 = make_gpu(c.leaves, c.weights, K, "f64")
    ref64.set_reversible(c.rates, c.pi)
    if K > 1:
        ref64.set_gamma(alpha)
    ref64.propose_lengths(internals, children, lengths, 1.0)
    g.propose_lengths(internals, children, lengths, 1.0)
    assert g.log_likelihood() == pytest.approx(ref64.log_likelihood(), rel=F32_TOL)
    g.close()
    ref64.close()
    return out


@pytest.mark.parametrize("K,alpha,taxa,sites", [(4, 0.5, 200, 6000), (1, None, 120, 3000),
                                                (3, 1.3, 90, 2500)])
def test_every_shape_gives_the_same_values(K, alpha, taxa, sites, monkeypatch):
    c = dna_case(taxa, sites, seed=80 + K, model="gtr", root_height=1.0, alpha=alpha,
                 num_categories=K, gaps=0.03, ambiguous=0.01)
    runs = {s: run_sequence(c, K, alpha, s, monkeypatch, seed=5) for s in SHAPES}
    base = runs[SHAPES[0]]
    for shape, seq in runs.items():
        assert len(seq) == len(base)
        for (lnl, site), (lnl0, site0) in zip(seq, base):
            assert np.array_equal(site, site0), shape
            assert lnl == pytest.approx(lnl0, rel=1e-13), shape
    # one (tile, block) shape: slots and inline tables change no bit
    for shape, seq in runs.items():
        twin = (SHAPES[0][0], SHAPES[0][1], 0, 0)
        if shape[:2] == twin[:2]:
            assert [x[0] for x in seq] == [x[0] for x in base], shape


@pytest.mark.parametrize("precision,inline,want", [("f32", 1, 1), ("f32", 0, 2), ("f64", 1, 2)])
def test_kernels_per_evaluation(precision, inline, want, monkeypatch):
    """One launch for a run walk that builds its own tables, tables +
    pruning otherwise, one fused launch for a short FP32 list."""
    monkeypatch.setenv("B3G_RUNS_INLINE", str(inline))
    c = dna_case(64, 2000, seed=91, model="gtr", alpha=0.5, num_categories=4)
    g = make_gpu(c.leaves, c.weights, 4, precision)
    g.set_reversible(c.rates, c.pi)
    g.set_gamma(0.5)
    tree = full(c.tree.parents, c.tree.heights)
    g.propose_lengths(*lists_and_lengths(tree), 1.0)
    g.log_likelihood()
    assert g.last_launches() == want
    g.accept()
    tree.accept()
    random_move(tree, np.random.default_rng(3))
    internals, children, lengths = lists_and_lengths(tree)
    g.propose_lengths(internals, children, lengths, 1.0)
    g.log_likelihood()
    if precision == "f32" and len(internals) <= 48:
        assert g.last_launches() == 1
    g.close()

"""The tree operators of the native MCMC driver sample the Yule prior.

Every tip of a 5-taxon alignment is unknown, so every partial is one and the
likelihood is zero (to FP32 rounding, a few 1e-6 in all, far too little to
move an acceptance): the chain targets the prior alone.  Under the Yule
density the driver uses (priors/yule.rs:23-40), the coalescence intervals of
a 5-taxon tree with birth rate lambda are independent exponentials of rates
5, 4, 3 and 2 times lambda, so

- lambda * root height has mean 1/5 + 1/4 + 1/3 + 1/2 = 1.28333 whatever
  lambda is;
- every ranked labelled history is equally likely, so a labelled topology's
  probability is proportional to its number of rankings: caterpillars (60
  labelled topologies, one ranking each) 1/3, ((2,1),2) shapes (30, three
  rankings) 1/2, ((2,2),1) shapes (15, two rankings) 1/6.

The first test runs SubtreeSlide and BeastNarrowExchange alone.  It pins the
Hastings term of SubtreeSlide's downward topology change, +log of the number
of destinations: with the reference's -log (_subtree_slide.py:94) the same
chain's mean root height comes out near 1.39-1.45 instead of 1.283 (a pure
Python restatement of this chain, 3-4e5 steps, shows it), while the shape
frequencies barely move.  The second adds NodeSlide, RootSlide, TreeScale,
BeastWideExchange, UpDown(tree, birth rate) and the birth-rate scale, with
the birth rate free under its LogNormal(1, 1.5) prior, whose marginal it
keeps because the Yule density integrates to the same constant for every
lambda.  Means are compared within 4.5 standard errors from the effective
sample size (Geyer 1992); operators are not tuned during these runs, so each
chain is exactly reversible.
"""

import numpy as np
import pytest

from aspartik_gb300.ess import ess
from tests.cases import dna_case

pytestmark = pytest.mark.gpu

ROOT_SCALED_MEAN = 1 / 5 + 1 / 4 + 1 / 3 + 1 / 2
SHAPES = {"caterpillar": 1 / 3, "3+2": 1 / 2, "4+1 balanced": 1 / 6}


def shape(parents: np.ndarray, L: int) -> str:
    """Shape class of a 5-taxon rooted tree from its parent array."""
    n = parents.size
    size = np.zeros(n, dtype=np.int64)
    size[:L] = 1
    for v in range(L):  # every leaf counts in each of its ancestors
        u = int(parents[v])
        while u != 0xFFFFFFFF:
            size[u] += 1
            u = int(parents[u])
    inner = sorted(int(size[v]) for v in range(L, n) if parents[v] != 0xFFFFFFFF)
    return {(2, 3, 4): "caterpillar", (2, 2, 3): "3+2", (2, 2, 4): "4+1 balanced"}[tuple(inner)]


def run_prior_chain(weights, steps, seed, birth_rate=1.0):
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    c = dna_case(5, 20, seed=seed)
    c.leaves = np.full_like(c.leaves, 0x0F)  # every tip unknown
    s = McmcSettings(model="hky", precision="f32", num_categories=1, sample_every=10,
                     tune_every=0, seed=seed, weights=weights)
    m = Mcmc(c.leaves, c.weights, c.tree.parents, c.tree.heights, s)
    m.set_parameters(kappa=2.0, frequencies=np.full(4, 0.25), birth_rate=birth_rate)
    m.run(steps)
    assert abs(m.trace("lnl")).max() < 1e-4
    smp = m.samples()
    stats = m.operator_stats()
    m.close()
    return smp, stats


def check_mean(x, want, label):
    x = np.asarray(x, dtype=np.float64)
    n_eff = ess(x, burn_in=0.0)
    assert n_eff > 200, (label, n_eff)
    se = x.std() / np.sqrt(n_eff)
    assert abs(x.mean() - want) < 4.5 * se, (label, x.mean(), want, se, n_eff)


def check_shapes(parents, L=5):
    shapes = [shape(p, L) for p in parents]
    for name, prob in SHAPES.items():
        check_mean([s == name for s in shapes], prob, name)


def root_heights(smp):
    return np.array([h[p == 0xFFFFFFFF][0] for h, p in zip(smp["heights"], smp["parents"])])


def test_subtree_slide_and_narrow_exchange_sample_the_yule_prior():
    smp, stats = run_prior_chain(dict(subtree_slide=1.0, narrow_exchange=1.0), 1_000_000,
                                 seed=21)
    keep = slice(smp["step"].size // 20, None)
    check_mean(root_heights(smp)[keep], ROOT_SCALED_MEAN, "root height")
    check_shapes(smp["parents"][keep])
    assert stats["subtree_slide"]["accepts"] > 10_000
    assert stats["narrow_exchange"]["accepts"] > 10_000


def test_height_operators_sample_the_yule_prior():
    weights = dict(subtree_slide=3.0, narrow_exchange=3.0, node_slide=3.0, root_slide=1.0,
                   tree_scale=1.0, wide_exchange=1.0, up_down=1.0, scale_birth_rate=1.0)
    smp, stats = run_prior_chain(weights, 1_000_000, seed=22, birth_rate=2.0)
    keep = slice(smp["step"].size // 20, None)
    lam = smp["birth_rate"]
    check_mean((lam * root_heights(smp))[keep], ROOT_SCALED_MEAN, "birth rate x root height")
    check_mean(np.log(lam)[keep], 1.0, "log birth rate")
    check_shapes(smp["parents"][keep])
    for name in weights:
        assert stats[name]["accepts"] > 1_000, (name, stats[name])

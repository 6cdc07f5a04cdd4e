"""Site-pattern compression on the device against the oracle's
deduplicate (likelihood/mod.rs:74-132): bit-exact leaves, weights and
site-to-pattern maps."""

import numpy as np
import pytest

from aspartik_gb300 import sim
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def gpu_dedup(msa, dna=True):
    from aspartik_gb300.calculator import deduplicate

    return deduplicate(msa, dna=dna)


def check(msa):
    leaves, weights, s2p, _ = gpu_dedup(msa)
    ol, ow, os_ = O.deduplicate(msa)
    np.testing.assert_array_equal(leaves, ol)
    np.testing.assert_array_equal(weights, ow)
    np.testing.assert_array_equal(s2p, os_)
    assert int(weights.sum()) == msa.shape[1]


def test_random_dna_with_gaps_and_repeats(rng):
    # few distinct columns: many repeats
    base = sim.random_dna(12, 40, rng)
    msa = base[:, rng.integers(0, 40, size=3000)]
    msa[rng.random(msa.shape) < 0.03] = 0
    check(np.ascontiguousarray(msa))


def test_simulated_alignment_full_size(rng):
    tree = sim.yule_tree(200, rng, root_height=0.3)
    pi = sim.dirichlet([5.0] * 4, rng)
    Q = sim.reversible_q(rng.gamma(2.0, 1.0, 6), pi)
    states = sim.simulate_alignment(tree, 50000, Q, pi, rng)
    check(sim.to_dna_codes(states))


@pytest.mark.parametrize("shape", [(2, 1), (1, 7), (5, 1000), (3, 64)])
def test_edge_shapes(shape, rng):
    L, N = shape
    msa = sim.random_dna(L, N, rng)
    check(msa)


def test_all_identical_and_all_distinct(rng):
    col = sim.random_dna(9, 1, rng)
    check(np.ascontiguousarray(np.repeat(col, 777, axis=1)))
    # 4^6 = 4096 distinct columns, each once, shuffled
    codes = np.array([1, 2, 4, 8], dtype=np.uint8)
    grid = np.array(np.meshgrid(*[np.arange(4)] * 6, indexing="ij")).reshape(6, -1)
    msa = codes[grid][:, rng.permutation(grid.shape[1])]
    check(np.ascontiguousarray(msa))


def test_protein_codes_are_kept(rng):
    msa = rng.integers(0, 21, size=(7, 2000)).astype(np.uint8)
    leaves, weights, s2p, _ = gpu_dedup(msa, dna=False)
    ref_leaves, ref_w, ref_s2p = sim.deduplicate(msa, dna=False)
    np.testing.assert_array_equal(leaves, ref_leaves)
    np.testing.assert_array_equal(weights, ref_w)
    np.testing.assert_array_equal(s2p, ref_s2p)

"""Generates tests/golden/small_trees.npz.

These golden vectors are ground truth computed independently of any pruning
code (values produced by the reference itself, by its FP64 CUDA kernel, are
in ref_cuda_partials.npz, made by make_ref_cuda_golden.py): brute-force enumeration of internal states with P(t) from
scipy's matrix exponential, summed in longdouble (oracle/brute.py).  Inputs
are seeded and small enough to regenerate in seconds.

Run: python tests/golden/make_golden.py
"""

from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from aspartik_gb300 import sim  # noqa: E402
from oracle import brute  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_trees.npz")

# (name, taxa, sites, model, alpha, categories, gap fraction, ambiguous fraction, root height)
CASES = [
    ("jc_2taxa", 2, 40, "jc", None, 1, 0.0, 0.0, 0.3),
    ("hky_4taxa", 4, 60, "hky", None, 1, 0.0, 0.0, 0.5),
    ("gtr_5taxa_gaps", 5, 80, "gtr", None, 1, 0.1, 0.05, 0.8),
    ("hky_6taxa_deep", 6, 50, "hky", None, 1, 0.0, 0.0, 3.0),
    ("gtr_g4_5taxa", 5, 60, "gtr", 0.5, 4, 0.05, 0.0, 1.0),
    ("hky_g2_4taxa", 4, 40, "hky", 1.5, 2, 0.0, 0.1, 0.4),
]


def main() -> None:
    data = {}
    for i, (name, L, N, model, alpha, K, gaps, amb, rh) in enumerate(CASES):
        rng = np.random.default_rng(4 + i)
        tree = sim.yule_tree(L, rng, root_height=rh)
        if model == "jc":
            pi = np.full(4, 0.25)
            rates = np.ones(6)
        elif model == "hky":
            pi = sim.dirichlet([10.0] * 4, rng)
            rates = sim.hky_rates(2.0)
        else:
            pi = sim.dirichlet([5.0] * 4, rng)
            rates = rng.gamma(2.0, 1.0, size=6)
        Q = sim.reversible_q(rates, pi)
        cats = sim.gamma_rates(alpha, K) if alpha is not None else np.ones(1)
        states = sim.simulate_alignment(tree, N, Q, pi, rng, cat_rates=cats)
        msa = sim.to_dna_codes(states)
        if gaps:
            msa[rng.random(msa.shape) < gaps] = 0
        if amb:
            m = rng.random(msa.shape) < amb
            msa[m] = rng.choice(np.array([3, 5, 15], dtype=np.uint8), size=m.sum())
        leaves, weights, _ = sim.deduplicate(msa)
        site = brute.site_log_likelihoods(tree.parents, tree.heights, leaves, Q, pi,
                                          cat_rates=cats)
        total = np.sum(site * weights.astype(np.longdouble))
        p = f"{name}/"
        data[p + "parents"] = tree.parents
        data[p + "heights"] = tree.heights
        data[p + "pi"] = pi
        data[p + "rates"] = rates
        data[p + "alpha"] = np.array(np.nan if alpha is None else alpha)
        data[p + "categories"] = np.array(K)
        data[p + "cat_rates"] = cats
        data[p + "leaves"] = leaves
        data[p + "weights"] = weights
        data[p + "site_lnl"] = site.astype(np.float64)
        data[p + "lnl"] = np.array(float(total))
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({len(CASES)} cases)")


if __name__ == "__main__":
    main()

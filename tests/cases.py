"""Seeded problem instances shared by the tests."""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from aspartik_gb300 import sim


@dataclass
class Case:
    tree: sim.Tree
    pi: np.ndarray
    rates: np.ndarray   # exchangeabilities (GTR order), or None for HKY
    kappa: float | None
    leaves: np.ndarray  # [L][P] IUPAC codes
    weights: np.ndarray
    msa: np.ndarray     # [L][N] raw codes before deduplication


def dna_case(num_leaves: int, num_sites: int, seed: int = 4, model: str = "hky",
             root_height: float = 0.5, alpha: float | None = None, num_categories: int = 1,
             gaps: float = 0.0, ambiguous: float = 0.0, pi_conc: float = 10.0) -> Case:
    rng = np.random.default_rng(seed)
    tree = sim.yule_tree(num_leaves, rng, root_height=root_height)
    pi = sim.dirichlet([pi_conc] * 4, rng)
    if model == "hky":
        kappa = 2.0
        rates = sim.hky_rates(kappa)
    else:
        kappa = None
        rates = rng.gamma(2.0, 1.0, size=6)
    Q = sim.reversible_q(rates, pi)
    cats = sim.gamma_rates(alpha, num_categories) if alpha is not None else None
    states = sim.simulate_alignment(tree, num_sites, Q, pi, rng, cat_rates=cats)
    msa = sim.to_dna_codes(states)
    if gaps:
        msa[rng.random(msa.shape) < gaps] = 0
    if ambiguous:
        amb = rng.random(msa.shape) < ambiguous
        msa[amb] = rng.choice(np.array([3, 5, 6, 9, 10, 12, 15], dtype=np.uint8), size=amb.sum())
    leaves, weights, _ = sim.deduplicate(msa)
    return Case(tree, pi, None if model == "hky" else rates, kappa, leaves, weights, msa)


def protein_case(num_leaves: int, num_sites: int, seed: int = 4, root_height: float = 1.0,
                 alpha: float | None = 1.0, num_categories: int = 4,
                 gaps: float = 0.0) -> Case:
    """20 states: exchangeabilities r_ij ~ LogNormal(0, 1) (190 values,
    upper-triangle row-major), pi ~ Dir(1 x 20), Yule tree, Gamma categories;
    codes are state indices 0..19 and 255 marks a gap (unknown)."""
    rng = np.random.default_rng(seed)
    tree = sim.yule_tree(num_leaves, rng, root_height=root_height)
    pi = sim.dirichlet([1.0] * 20, rng)
    pi = np.maximum(pi, 1e-4)
    pi /= pi.sum()
    rates = rng.lognormal(0.0, 1.0, size=190)
    Q = sim.reversible_q(rates, pi)
    cats = sim.gamma_rates(alpha, num_categories) if alpha is not None else None
    states = sim.simulate_alignment(tree, num_sites, Q, pi, rng, cat_rates=cats)
    if gaps:
        states[rng.random(states.shape) < gaps] = 255
    leaves, weights, _ = sim.deduplicate(states, dna=False)
    return Case(tree, pi, rates, None, leaves, weights, states)

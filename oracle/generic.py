"""Generic-S pruning oracle.  TEST INFRASTRUCTURE ONLY.

The checker for the 20-state (protein) GPU path: it is called from tests/,
never from the product path.  It restates the reference's CPU pruner
(crates/b3/src/calculator/cpu4.rs:170-433) with S states instead of 4, in
numpy FP64:

  - a tip child contributes the column P[:, code] of its edge's transition
    matrix, or 1.0 for an unknown code (cpu4.rs:117-124, 288-360; here a
    code >= S is unknown);
  - an internal child contributes P x (cpu4.rs:361-401);
  - a node whose S entries are all below e^-scale_ln is multiplied by
    e^scale_ln and counted, except tip-tip nodes (cpu4.rs:288-318, 403-433);
  - the root gives ln(pi . x) - count * scale_ln (cpu4.rs:277-284);
  - Gamma categories mix by log-sum-exp plus ln(1/K) and the patterns are
    weighted (gamma.rs:97-169, likelihood/mod.rs:134-151).

Parity status: for S = 20 unpinned against outputs of the reference itself
(the reference has no 20-state calculator; its GenericSubstitution is not
used by one).  Pinned here against the 4-state restatement (the S = 4 case
must agree with cpu4, which in turn reproduces the reference's own FP64 CUDA
kernel, tests/test_ref_golden.py), the JC-20 closed form and brute-force
enumeration.
"""

from __future__ import annotations

import numpy as np

from . import oracle as O


def prune(leaves: np.ndarray, internals, children, matrices: np.ndarray,
          pi: np.ndarray, scale_ln: int = 30) -> np.ndarray:
    """Per-pattern lnL of one category.  leaves [L][P] state codes (>= S is
    unknown); matrices [n][2][S][S] row-major P of each listed internal's
    left and right child edge; the list is children-first, root last."""
    leaves = np.asarray(leaves)
    pi = np.asarray(pi, dtype=np.float64)
    S = pi.size
    L, P = leaves.shape
    thr, mult = np.exp(-float(scale_ln)), np.exp(float(scale_ln))
    partial, count = {}, {}
    for i, v in enumerate(internals):
        parts, tips = [], []
        cnt = np.zeros(P, dtype=np.int64)
        for side in range(2):
            ch = int(children[i][side])
            Pm = np.asarray(matrices[i][side], dtype=np.float64)
            if ch < L:
                codes = leaves[ch].astype(np.int64)
                known = codes < S
                col = np.ones((P, S))
                col[known] = Pm[:, codes[known]].T
                parts.append(col)
                tips.append(True)
            else:
                parts.append(partial[ch] @ Pm.T)
                cnt += count[ch]
                tips.append(False)
        y = parts[0] * parts[1]
        if not all(tips):
            small = (y < thr).all(axis=1)
            y[small] *= mult
            cnt += small
        partial[int(v)], count[int(v)] = y, cnt
    root = int(internals[-1])
    with np.errstate(divide="ignore"):
        return np.log(partial[root] @ pi) - count[root].astype(np.float64) * scale_ln


def lists(parents, heights):
    """Whole-tree children-first lists (tree.rs:423-461) with edge lengths."""
    t = O.DatedTree(parents, heights)
    t.mark_all_edges_updated()
    internals, children = t.partials_lists()
    lengths = np.array([[t.edge_length(int(a)), t.edge_length(int(b))]
                        for a, b in children]).reshape(-1, 2)
    return internals, children, lengths


def site_log_likelihoods(leaves, parents, heights, model: O.EigenModel,
                         cat_rates=None, clock_rate: float = 1.0,
                         scale_ln: int = 30) -> np.ndarray:
    """Category-mixed per-pattern lnL of a whole tree."""
    internals, children, lengths = lists(parents, heights)
    cats = np.ones(1) if cat_rates is None else np.asarray(cat_rates, dtype=np.float64)
    per = []
    for r in cats:
        mats = np.array([[model.transition(d * clock_rate * r) for d in pair]
                         for pair in lengths])
        per.append(prune(leaves, internals, children, mats, model.pi, scale_ln))
    per = np.array(per)
    mx = per.max(axis=0)
    with np.errstate(invalid="ignore"):
        site = mx + np.log(np.exp(per - mx).sum(axis=0)) + np.log(1.0 / len(cats))
    return np.where(np.isfinite(mx), site, -np.inf)


def log_likelihood(leaves, weights, parents, heights, model: O.EigenModel,
                   cat_rates=None, clock_rate: float = 1.0, scale_ln: int = 30) -> float:
    site = site_log_likelihoods(leaves, parents, heights, model, cat_rates,
                                clock_rate, scale_ln)
    return float(site @ np.asarray(weights, dtype=np.float64))

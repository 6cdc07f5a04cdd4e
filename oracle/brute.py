"""Brute-force likelihood of small trees.  TEST INFRASTRUCTURE ONLY.

An independent ground truth for the pruning oracle and the GPU path: the
site likelihood is the sum, over every assignment of states to the internal
nodes, of pi(root state) times the product over edges of P(t)[parent state,
child state], with P(t) = expm(Q t) from scipy.  Tips with a single-base
code fix the child state; any other code is "unknown" and contributes 1, as
calculator/cpu4.rs:117-124 maps them.  With S != 4 states the codes are
state indices and a code >= S is unknown.  Sums run in numpy's longdouble.
"""

from __future__ import annotations

import itertools

import numpy as np
from scipy.linalg import expm

TOMBSTONE = 0xFFFFFFFF
_CODE_STATE = {1: 0, 2: 1, 4: 2, 8: 3}


def _state(code, S):
    if S == 4:
        return _CODE_STATE.get(int(code))
    return int(code) if int(code) < S else None


def site_log_likelihoods(parents, heights, leaves, Q, pi, cat_rates=None,
                         clock_rate=1.0) -> np.ndarray:
    parents = np.asarray(parents, dtype=np.int64)
    heights = np.asarray(heights, dtype=np.float64)
    leaves = np.asarray(leaves)
    Q = np.asarray(Q, dtype=np.float64)
    pi = np.asarray(pi, dtype=np.float64)
    S = pi.size
    n = parents.size
    L = (n + 1) // 2
    P_sites = leaves.shape[1]
    cats = np.ones(1) if cat_rates is None else np.asarray(cat_rates, dtype=np.float64)
    internals = list(range(L, n))
    root = int(np.nonzero(parents == TOMBSTONE)[0][0])
    total = np.zeros(P_sites, dtype=np.longdouble)
    for r in cats:
        mats = {}
        for v in range(n):
            if parents[v] == TOMBSTONE:
                continue
            t = (heights[parents[v]] - heights[v]) * (clock_rate * r)
            mats[v] = expm(Q * t).astype(np.longdouble)
        cat_lik = np.zeros(P_sites, dtype=np.longdouble)
        for assign in itertools.product(range(S), repeat=len(internals)):
            state = dict(zip(internals, assign))
            w = np.full(P_sites, np.longdouble(pi[state[root]]))
            for v in internals:
                if v == root:
                    continue
                w = w * mats[v][state[parents[v]], state[v]]
            for leaf in range(L):
                Pm = mats[leaf][state[parents[leaf]]]
                col = np.array([Pm[st] if st is not None else 1.0
                                for st in (_state(c, S) for c in leaves[leaf])],
                               dtype=np.longdouble)
                w = w * col
            cat_lik += w
        total += cat_lik / len(cats)
    return np.log(total)

"""Seeded synthetic data: Yule trees, substitution models and alignments.

The reference only generates i.i.d. random alignments
(crates/data/src/msa/mod.rs:183-191); benchmarks and tests here need
alignments with phylogenetic signal of a stated shape, so this module
simulates them.  Everything is driven by ``numpy.random.Generator`` seeded by
the caller (base seed 4, the reference's convention in
python/tests/conftest.py).

Trees use the reference's node numbering (parameters/tree.rs): leaves
0..L-1, internals L..2L-2, ``parents[root] == TOMBSTONE``.  Internals are
numbered in the order they are created going back in time, so every parent
has a larger id than its children and the root is 2L-2.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

TOMBSTONE = 0xFFFFFFFF
# IUPAC bit codes of A, C, G, T (crates/data/src/nucleotides.rs:50-71)
DNA_CODES = np.array([1, 2, 4, 8], dtype=np.uint8)


@dataclass
class Tree:
    parents: np.ndarray  # u32 [2L-1]
    heights: np.ndarray  # f64 [2L-1]

    @property
    def num_leaves(self) -> int:
        return (self.parents.size + 1) // 2

    @property
    def root(self) -> int:
        return int(np.nonzero(self.parents == TOMBSTONE)[0][0])

    def children(self) -> np.ndarray:
        """[I][2] children of each internal in the order load_parents fills
        them (parameters/tree.rs:906-930)."""
        L = self.num_leaves
        ch = np.full((L - 1, 2), TOMBSTONE, dtype=np.uint32)
        for node, par in enumerate(self.parents):
            if par == TOMBSTONE:
                continue
            k = int(par) - L
            if ch[k, 0] == TOMBSTONE:
                ch[k, 0] = node
            else:
                ch[k, 1] = node
        return ch


def yule_tree(num_leaves: int, rng: np.random.Generator, birth_rate: float = 1.0,
              root_height: float | None = None) -> Tree:
    """A Yule (pure-birth) tree: going back in time, k lineages merge after an
    Exp(k * birth_rate) wait, a uniformly random pair at a time.  With
    ``root_height`` the heights are rescaled so the root sits there."""
    L = int(num_leaves)
    if L < 2:
        raise ValueError("a tree needs at least two leaves")
    parents = np.full(2 * L - 1, TOMBSTONE, dtype=np.uint32)
    heights = np.zeros(2 * L - 1, dtype=np.float64)
    lineages = list(range(L))
    t = 0.0
    nxt = L
    while len(lineages) > 1:
        k = len(lineages)
        t += rng.exponential(1.0 / (k * birth_rate))
        i, j = rng.choice(k, size=2, replace=False)
        a, b = lineages[i], lineages[j]
        for idx in sorted((i, j), reverse=True):
            lineages.pop(idx)
        parents[a] = nxt
        parents[b] = nxt
        heights[nxt] = t
        lineages.append(nxt)
        nxt += 1
    if root_height is not None:
        heights *= root_height / heights[2 * L - 2]
    return Tree(parents, heights)


def dirichlet(alpha, rng: np.random.Generator) -> np.ndarray:
    return rng.dirichlet(np.asarray(alpha, dtype=np.float64))


def reversible_q(rates: np.ndarray, pi: np.ndarray) -> np.ndarray:
    """Q_ij = r_ij pi_j from symmetric exchangeabilities in upper-triangle
    row-major order, normalised to mean rate 1."""
    n = pi.size
    Q = np.zeros((n, n))
    iu = np.triu_indices(n, 1)
    R = np.zeros((n, n))
    R[iu] = rates
    R = R + R.T
    Q = R * pi[None, :]
    np.fill_diagonal(Q, 0.0)
    np.fill_diagonal(Q, -Q.sum(axis=1))
    return Q / -(np.diag(Q) @ pi)


def hky_rates(kappa: float) -> np.ndarray:
    """HKY as GTR exchangeabilities (AC, AG, AT, CG, CT, GT)."""
    return np.array([1.0, kappa, 1.0, 1.0, kappa, 1.0])


def transition_matrices(Q: np.ndarray, pi: np.ndarray, ts: np.ndarray) -> np.ndarray:
    """P(t) = exp(Q t) for every t in ts through the symmetric eigensystem."""
    sq = np.sqrt(pi)
    B = sq[:, None] * Q / sq[None, :]
    B = 0.5 * (B + B.T)
    lam, U = np.linalg.eigh(B)
    V = U / sq[:, None]
    Vi = U.T * sq[None, :]
    e = np.exp(np.multiply.outer(np.asarray(ts, dtype=np.float64), lam))
    P = np.einsum("ik,tk,kj->tij", V, e, Vi)
    return np.clip(P, 0.0, None)


def gamma_rates(alpha: float, k: int) -> np.ndarray:
    """Median-discretised Gamma categories normalised to mean 1
    (likelihood/gamma.rs:205-225), from scipy's inverse incomplete gamma."""
    from scipy.special import gammaincinv

    q = gammaincinv(alpha, (2.0 * np.arange(k) + 1.0) / (2.0 * k))
    return q / q.mean()


def simulate_alignment(tree: Tree, num_sites: int, Q: np.ndarray, pi: np.ndarray,
                       rng: np.random.Generator, cat_rates: np.ndarray | None = None,
                       clock_rate: float = 1.0) -> np.ndarray:
    """States [L][num_sites] (0..S-1) evolved down ``tree`` under Q; each site
    draws a rate category uniformly from ``cat_rates``."""
    S = pi.size
    L = tree.num_leaves
    n = tree.parents.size
    cat_rates = np.ones(1) if cat_rates is None else np.asarray(cat_rates, dtype=np.float64)
    site_cat = rng.integers(0, cat_rates.size, size=num_sites)
    states = np.zeros((n, num_sites), dtype=np.int64)
    root = tree.root
    states[root] = rng.choice(S, size=num_sites, p=pi)
    # parents have larger ids than their children: visit ids downwards
    for node in range(n - 1, -1, -1):
        par = tree.parents[node]
        if par == TOMBSTONE:
            continue
        t = (tree.heights[par] - tree.heights[node]) * clock_rate
        Ps = transition_matrices(Q, pi, t * cat_rates)  # [K][S][S]
        cdf = np.cumsum(Ps, axis=2)
        cdf[:, :, -1] = 1.0
        rows = cdf[site_cat, states[par]]  # [sites][S]
        u = rng.random(num_sites)
        states[node] = (u[:, None] > rows).sum(axis=1)
    return states[:L].astype(np.uint8)


def to_dna_codes(states: np.ndarray) -> np.ndarray:
    return DNA_CODES[states]


def random_dna(num_sequences: int, num_sites: int, rng: np.random.Generator) -> np.ndarray:
    """i.i.d. uniform bases, as Msa::random (crates/data/src/msa/mod.rs:183-191)."""
    return DNA_CODES[rng.integers(0, 4, size=(num_sequences, num_sites))]


def deduplicate(msa: np.ndarray, dna: bool = True):
    """Site-pattern compression (likelihood/mod.rs:74-132): unique columns in
    first-occurrence order, their counts, the pattern of every site, and the
    leaf-major pattern matrix.  For DNA (IUPAC codes) gaps (code 0) map to
    0b1111; for protein state indices (dna=False) codes are kept as given."""
    msa = np.ascontiguousarray(msa, dtype=np.uint8)
    L, N = msa.shape
    cols = np.ascontiguousarray(msa.T)
    view = cols.view(np.dtype((np.void, L))).reshape(N)
    _, first, inverse, counts = np.unique(view, return_index=True, return_inverse=True,
                                          return_counts=True)
    order = np.argsort(first, kind="stable")  # first-occurrence order
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    leaves = msa[:, first[order]].copy()
    if dna:
        leaves[leaves == 0] = 0x0F
    weights = counts[order].astype(np.uint32)
    site_to_pattern = rank[inverse.reshape(-1)].astype(np.uint32)
    return leaves, weights, site_to_pattern
